// hydro_adjoint.cuh -- reverse-mode (adjoint) rules of the examples/Hydro
// scheme pieces in hydro_scheme.cuh.  Each *_rev function recomputes what it
// needs of its forward and adds input cotangents (accumulating with +=) from
// output cotangents.  Branch decisions (HLLC case, minmod pick, max clamps,
// hllcQ case, CFL min) are those of the forward; the derivative follows the
// branch taken, as finite differences do away from the switching points.
#pragma once

#include "hydro_scheme.cuh"

namespace om {
namespace ha {

using hs::Flux;
using hs::Prim;

// cotangents of a primitive record
template <class R> struct PrimBar {
  R rho, v0, v1, p;
};

template <class R> __device__ __forceinline__ void zero(PrimBar<R> &a) {
  a.rho = a.v0 = a.v1 = a.p = R(0);
}

// c = sqrt(g p / rho): cotangent cb -> (rho, p)
template <class R>
__device__ __forceinline__ void sound_rev(R g, R rho, R p, R c, R cb, R &rhob, R &pb) {
  if (cb == R(0)) return;
  const R tb = R(0.5) * cb / c;
  const R gr = g / rho;
  pb += tb * gr;
  rhob -= tb * gr * p / rho;
}

// kinetic energy 0.5 (v0 m0 + v1 m1)
template <class R>
__device__ __forceinline__ void kinetic_rev(R v0, R v1, R m0, R m1, R keb, R &v0b, R &v1b,
                                            R &m0b, R &m1b) {
  const R h = R(0.5) * keb;
  v0b += h * m0;
  v1b += h * m1;
  m0b += h * v0;
  m1b += h * v1;
}

// flux_prim<AX> reverse: fb -> (rho, v0, v1, p)
template <int AX, class R>
__device__ __forceinline__ void flux_prim_rev(const hf::Consts<R> &k, R rho, R v0, R v1, R p,
                                              const Flux<R> &fb, PrimBar<R> &xb) {
  const R m0 = rho * v0, m1 = rho * v1;
  const R e = hs::kinetic(v0, v1, m0, m1) + k.gm1inv * p;
  const R h = e + p;
  const R va = AX == 0 ? v0 : v1;
  R m0b = 0, m1b = 0, vab = 0, v0b = 0, v1b = 0, pb = 0;
  if (AX == 0) m0b += fb.fd; else m1b += fb.fd;
  m0b += fb.fm0 * va;
  m1b += fb.fm1 * va;
  vab += fb.fm0 * m0 + fb.fm1 * m1;
  pb += AX == 0 ? fb.fm0 : fb.fm1;
  const R hb = fb.fe * va;
  vab += fb.fe * h;
  const R eb = hb;
  pb += hb;
  pb += eb * k.gm1inv;
  kinetic_rev(v0, v1, m0, m1, eb, v0b, v1b, m0b, m1b);
  if (AX == 0) v0b += vab; else v1b += vab;
  xb.rho += m0b * v0 + m1b * v1;
  xb.v0 += v0b + m0b * rho;
  xb.v1 += v1b + m1b * rho;
  xb.p += pb;
}

// star_flux<AX> reverse: fb -> (sstar, shock, rho, v0, v1, p), in closed
// form.  The star record of side K (HydroMain.hs:272-282) is density
// d = rho (S - u) / (S - S*), velocity (S* along the wall, the side's own
// across it: what m/rho of the record recovers) and energy density
// d (E/rho + (S* - u)(S* + p/(rho (S - u)))); its pressure is the equation
// of state of the record, p* = (g-1)(e - d (S*^2 + vt^2)/2), and its flux
// (d S*, d S*^2 + p*, d vt S*, (e + p*) S*).  This is the derivative of the
// same function as the flux of the recovered record; three reciprocals.
template <int AX, class R>
__device__ __forceinline__ void star_flux_rev(const hf::Consts<R> &k, R sstar, R shock, R rho,
                                              R v0, R v1, R p, const Flux<R> &fb, R &sstarb,
                                              R &shockb, PrimBar<R> &xb) {
  const R gm1 = k.gm1, gm1inv = k.gm1inv;
  const R u = AX == 0 ? v0 : v1, vt = AX == 0 ? v1 : v0;
  const R fdb = fb.fd, fnb = AX == 0 ? fb.fm0 : fb.fm1, ftb = AX == 0 ? fb.fm1 : fb.fm0;
  const R su = shock - u, ss = shock - sstar;
  const R rss = R(1) / ss, rsu = R(1) / su, rr = R(1) / rho;
  const R dens = rho * su * rss;
  const R E = R(0.5) * rho * (u * u + vt * vt) + gm1inv * p;
  const R w = p * rr * rsu;
  const R z = sstar + w;
  const R y = (sstar - u) * z;
  const R x = E * rr + y;
  const R enrg = dens * x;
  const R q2 = sstar * sstar + vt * vt;
  const R pst = gm1 * (enrg - R(0.5) * dens * q2);
  // flux components
  R densb = fdb * sstar + fnb * sstar * sstar + ftb * vt * sstar;
  R Ssb = fdb * dens + fnb * R(2) * dens * sstar + ftb * dens * vt + fb.fe * (enrg + pst);
  R vtb = ftb * dens * sstar;
  R enrgb = fb.fe * sstar;
  const R pstb = fnb + fb.fe * sstar;
  // p* = (g-1)(e - d q2 / 2)
  enrgb += gm1 * pstb;
  densb -= gm1 * pstb * R(0.5) * q2;
  Ssb -= gm1 * pstb * dens * sstar;
  vtb -= gm1 * pstb * dens * vt;
  // e = d x, x = E/rho + (S* - u) z, z = S* + p/(rho (S - u))
  densb += enrgb * x;
  const R xbar = enrgb * dens;
  const R Eb = xbar * rr;
  R rrb = xbar * E;
  R ub = -xbar * z;
  Ssb += xbar * z;
  const R zb = xbar * (sstar - u);
  Ssb += zb;
  R pb = zb * rr * rsu;
  rrb += zb * p * rsu;
  R sub = -zb * w * rsu;
  R rhob = -rrb * rr * rr;
  // E = rho (u^2 + vt^2) / 2 + p/(g-1)
  rhob += Eb * R(0.5) * (u * u + vt * vt);
  ub += Eb * rho * u;
  vtb += Eb * rho * vt;
  pb += Eb * gm1inv;
  // d = rho (S - u) / (S - S*)
  rhob += densb * su * rss;
  sub += densb * rho * rss;
  const R ssb = -densb * dens * rss;
  shockb += sub + ssb;
  ub -= sub;
  sstarb += Ssb - ssb;
  xb.rho += rhob;
  if (AX == 0) {
    xb.v0 += ub;
    xb.v1 += vtb;
  } else {
    xb.v1 += ub;
    xb.v0 += vtb;
  }
  xb.p += pb;
}

// hllcQ reverse: cotangent of q = sqrt(t) -> (sp, p), t = 1 + qc (sp/p - 1)
// (qc = (g+1)/(2g)); q is the forward's value
template <class R>
__device__ __forceinline__ void hllc_q_rev(R qc, R sp, R p, R q, R qb, R &spb, R &pb) {
  if (p <= sp) return;  // constant branch
  const R rp = R(1) / p;
  const R tb = R(0.5) * qb / q;
  spb += tb * qc * rp;
  pb -= tb * qc * sp * rp * rp;
}

// hllc<AX> reverse: cotangent of the wall fluxes -> cotangents of the two
// primitive states (the sound speeds' dependence on them included).  The
// forward quantities are recomputed with the expressions of the production
// algebra (hf::hllc), so the branch decisions are the FP32 forward's; the
// derivative is that of the same function in either algebra.
template <int AX, class R>
__device__ __forceinline__ void hllc_rev(const hf::Consts<R> &k, const Prim<R> &L,
                                         const Prim<R> &Rt, const Flux<R> &fb, PrimBar<R> &Lb,
                                         PrimBar<R> &Rb) {
  const R g = k.g;
  const R cl = hs::sound(g, L.rho, L.p), cr = hs::sound(g, Rt.rho, Rt.p);
  const R densMid = R(0.5) * (L.rho + Rt.rho);
  const R soundMid = R(0.5) * (cl + cr);
  const R uL = AX == 0 ? L.v0 : L.v1;
  const R uR = AX == 0 ? Rt.v0 : Rt.v1;
  const R psraw = R(0.5) * (L.p + Rt.p) - densMid * soundMid * (uR - uL);
  const R presStar = hs::omax(R(0), psraw);
  const R tL = sqrt(R(1) + k.qc * (presStar / L.p - R(1)));
  const R tR = sqrt(R(1) + k.qc * (presStar / Rt.p - R(1)));
  const R qL = (L.p <= presStar) ? R(1) : tL;
  const R qR = (Rt.p <= presStar) ? R(1) : tR;
  const R shockLeft = uL - cl * qL;
  const R shockRight = uR + cr * qR;
  const R aL = L.rho * (shockLeft - uL), aR = Rt.rho * (shockRight - uR);
  const R num = Rt.p - L.p + aL * uL - aR * uR;
  const R rden = R(1) / (aL - aR);
  const R shockStar = num * rden;
  const bool posL = R(0) < shockLeft, posS = R(0) < shockStar, posR = R(0) < shockRight;
  const bool useL = posL || posS;
  const bool star = useL ? !posL : posR;
  const Prim<R> &X = useL ? L : Rt;
  PrimBar<R> &Xb = useL ? Lb : Rb;
  if (!star) {
    flux_prim_rev<AX>(k, X.rho, X.v0, X.v1, X.p, fb, Xb);
    return;
  }
  const R shock = useL ? shockLeft : shockRight;
  R sstarb = 0, shockb = 0;
  star_flux_rev<AX>(k, shockStar, shock, X.rho, X.v0, X.v1, X.p, fb, sstarb, shockb, Xb);
  R SLb = useL ? shockb : R(0), SRb = useL ? R(0) : shockb;
  R rhoLb = 0, rhoRb = 0, uLb = 0, uRb = 0, pLb = 0, pRb = 0, clb = 0, crb = 0;
  // shockStar = num / den, num = pR - pL + aL uL - aR uR, den = aL - aR
  const R numb = sstarb * rden;
  const R denb = -sstarb * shockStar * rden;
  pRb += numb;
  pLb -= numb;
  const R aLb = numb * uL + denb, aRb = -numb * uR - denb;
  uLb += numb * aL;
  uRb -= numb * aR;
  // aL = rhoL (SL - uL), aR = rhoR (SR - uR)
  rhoLb += aLb * (shockLeft - uL);
  SLb += aLb * L.rho;
  uLb -= aLb * L.rho;
  rhoRb += aRb * (shockRight - uR);
  SRb += aRb * Rt.rho;
  uRb -= aRb * Rt.rho;
  // shock speeds
  uLb += SLb;
  clb -= SLb * qL;
  const R qLb = -SLb * cl;
  uRb += SRb;
  crb += SRb * qR;
  const R qRb = SRb * cr;
  R psb = 0;
  hllc_q_rev(k.qc, presStar, L.p, tL, qLb, psb, pLb);
  hllc_q_rev(k.qc, presStar, Rt.p, tR, qRb, psb, pRb);
  const R psrawb = (R(0) < psraw) ? psb : R(0);
  pLb += R(0.5) * psrawb;
  pRb += R(0.5) * psrawb;
  const R dmb = -psrawb * soundMid * (uR - uL);
  const R smb = -psrawb * densMid * (uR - uL);
  uRb -= psrawb * densMid * soundMid;
  uLb += psrawb * densMid * soundMid;
  rhoLb += R(0.5) * dmb;
  rhoRb += R(0.5) * dmb;
  clb += R(0.5) * smb;
  crb += R(0.5) * smb;
  sound_rev(g, L.rho, L.p, cl, clb, rhoLb, pLb);
  sound_rev(g, Rt.rho, Rt.p, cr, crb, rhoRb, pRb);
  Lb.rho += rhoLb;
  Lb.p += pLb;
  Rb.rho += rhoRb;
  Rb.p += pRb;
  if (AX == 0) {
    Lb.v0 += uLb;
    Rb.v0 += uRb;
  } else {
    Lb.v1 += uLb;
    Rb.v1 += uRb;
  }
}

// minmod MUSCL reverse for one field: (lb, rb) -> x0..x3
template <class R>
__device__ __forceinline__ void muscl_rev(R x0, R x1, R x2, R x3, R lb, R rb, R &x0b, R &x1b,
                                          R &x2b, R &x3b) {
  const R d01 = x1 - x0, d12 = x2 - x1, d23 = x3 - x2;
  x1b += lb;
  x2b += rb;
  const R d1b = lb / R(2), d2b = -rb / R(2);
  R d01b = 0, d12b = 0, d23b = 0;
  if (!(d01 * d12 <= R(0))) {
    if (fabs(d01) < fabs(d12)) d01b += d1b; else d12b += d1b;
  }
  if (!(d12 * d23 <= R(0))) {
    if (fabs(d12) < fabs(d23)) d12b += d2b; else d23b += d2b;
  }
  x1b += d01b;
  x0b -= d01b;
  x2b += d12b;
  x1b -= d12b;
  x3b += d23b;
  x2b -= d23b;
}

// Conserved-state cotangent Ub (rho, m0, m1, E) of the update's output, from
// the primitive cotangent qb of update(): reverse of the clamps, velocity
// division and pressure recovery.  d2, b0, b1, e2: the new conserved state.
template <class R>
__device__ __forceinline__ void cons_from_prim_rev(R g, R d2, R b0, R b1, R e2,
                                                   const PrimBar<R> &qb, R Ub[4]) {
  const R rd = R(1) / d2;
  const R v0 = b0 * rd, v1 = b1 * rd;
  const R pn = (g - R(1)) * (e2 - hs::kinetic(v0, v1, b0, b1));
  R d2b = (R(1e-2) < d2) ? qb.rho : R(0);
  const R pnb = (R(1e-2) < pn) ? qb.p : R(0);
  R v0b = qb.v0, v1b = qb.v1, b0b = 0, b1b = 0;
  const R e2b = (g - R(1)) * pnb;
  const R keb = -(g - R(1)) * pnb;
  kinetic_rev(v0, v1, b0, b1, keb, v0b, v1b, b0b, b1b);
  b0b += v0b * rd;
  b1b += v1b * rd;
  d2b -= (v0b * v0 + v1b * v1) * rd;
  Ub[0] = d2b;
  Ub[1] = b0b;
  Ub[2] = b1b;
  Ub[3] = e2b;
}

// Reverse of the conserved record of a primitive base state, cons(b):
// Ub (rho, m0, m1, E) -> bb
template <class R>
__device__ __forceinline__ void cons_of_prim_rev(R g, const Prim<R> &b, const R Ub[4],
                                                 PrimBar<R> &bb) {
  const R m0 = b.rho * b.v0, m1 = b.rho * b.v1;
  R rhob = Ub[0], m0b = Ub[1], m1b = Ub[2], v0b = 0, v1b = 0;
  const R eb = Ub[3];
  bb.p += eb / (g - R(1));
  kinetic_rev(b.v0, b.v1, m0, m1, eb, v0b, v1b, m0b, m1b);
  rhob += m0b * b.v0 + m1b * b.v1;
  v0b += m0b * b.rho;
  v1b += m1b * b.rho;
  bb.rho += rhob;
  bb.v0 += v0b;
  bb.v1 += v1b;
}

// The update's new conserved state (d2, b0, b1, e2) before the primitive
// recovery, from the taped flux differences D (D[4 * axis + k], left wall -
// right wall), with the same operation order as hs::update
template <class R>
__device__ __forceinline__ void update_cons_d(R g, const Prim<R> &b, R dtdx0, R dtdx1,
                                              const R D[8], R out[4]) {
  const R m0 = b.rho * b.v0, m1 = b.rho * b.v1;
  const R e = hs::kinetic(b.v0, b.v1, m0, m1) + (R(1) / (g - R(1))) * b.p;
  const R d1 = b.rho + dtdx1 * D[4];
  const R a0 = m0 + dtdx1 * D[5];
  const R a1 = m1 + dtdx1 * D[6];
  const R e1 = e + dtdx1 * D[7];
  out[0] = d1 + dtdx0 * D[0];
  out[1] = a0 + dtdx0 * D[1];
  out[2] = a1 + dtdx0 * D[2];
  out[3] = e1 + dtdx0 * D[3];
}

// timescale reverse at one cell: tb -> (rho, v0, v1, p)
template <class R>
__device__ __forceinline__ void timescale_rev(R g, R dR0, R dR1, const Prim<R> &x, R tb,
                                              PrimBar<R> &xb) {
  const R c = hs::sound(g, x.rho, x.p);
  const R s0 = c + fabs(x.v0), s1 = c + fabs(x.v1);
  const R t0 = dR0 / s0, t1 = dR1 / s1;
  R cb = 0;
  if (t1 < t0) {
    const R s1b = -tb * t1 / s1;
    cb += s1b;
    xb.v1 += s1b * (x.v1 < R(0) ? R(-1) : R(1));
  } else {
    const R s0b = -tb * t0 / s0;
    cb += s0b;
    xb.v0 += s0b * (x.v0 < R(0) ? R(-1) : R(1));
  }
  sound_rev(g, x.rho, x.p, c, cb, xb.rho, xb.p);
}

}  // namespace ha
}  // namespace om

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
// tolerance.  Every operation is spelled out with its rounding (add, sub,
// mul and fma round to nearest, rcp and sqrt are the hardware
// approximations, subnormals flush to zero), in one template over the
// number type: a float, or a pair of floats (f2) that one packed f32x2
// instruction advances together.  So a kernel that evaluates two walls per
// thread with packed instructions and one that evaluates one wall per
// thread give the same bits.
//  * 1/(gamma-1) and (gamma+1)/(2 gamma) are formed once per launch;
//  * hllcQ = sqrt(1 + qc (p*/p - 1)) is taken as sqrt((1 - qc) + (qc/p) p*);
//  * S* = (pL - pR + mL uL + mR uR) / (mL + mR) with mL = rhoL cL qL and
//    mR = rhoR cR qR, i.e. the generated formula with aL = rhoL (SL - uL)
//    = -mL and aR = rhoR (SR - uR) = mR;
//  * the star state's flux is taken in closed form: its recovered velocity
//    is S* along the wall and the side's own velocity across it (m/rho of
//    the star record), its density r (S - u)/(S - S*) and its energy
//    density (E (S - u) + (S* - u)(r (S - u) S* + p)) / (S - S*), one
//    reciprocal for both; its pressure is the equation of state of the
//    star record, as bindConserved gives it (HydroMain.hs:272-282,
//    Hydro.hs:110-118);
//  * the physical and star fluxes share one flux formula applied to the
//    selected state (density, normal velocity, energy, pressure).
// The timescale and the MUSCL reconstruction stay those of hs:: (the reverse
// sweep recomputes both and must find the forward's values; the
// reconstruction's values are exact selections and halvings, the same in
// any spelling).
// ---------------------------------------------------------------------------
namespace hf {

using hs::Flux;
using hs::Prim;
using hs::omax;

// a pair of floats in one 64-bit register pair, and a pair of predicates
struct f2 {
  unsigned long long v;
};
struct m2 {
  bool x, y;
};

__device__ __forceinline__ f2 pack(float a, float b) {
  f2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void unpack(f2 r, float &a, float &b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r.v));
}

__device__ __forceinline__ float add(float a, float b) {
  float d;
  asm("add.rn.ftz.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
  return d;
}
__device__ __forceinline__ float sub(float a, float b) {
  float d;
  asm("sub.rn.ftz.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
  return d;
}
__device__ __forceinline__ float mul(float a, float b) {
  float d;
  asm("mul.rn.ftz.f32 %0, %1, %2;" : "=f"(d) : "f"(a), "f"(b));
  return d;
}
// a * b + c, one rounding
__device__ __forceinline__ float fma(float a, float b, float c) {
  float d;
  asm("fma.rn.ftz.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float rcp(float a) {
  float d;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(d) : "f"(a));
  return d;
}
__device__ __forceinline__ float sqrt_(float a) {
  float d;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(d) : "f"(a));
  return d;
}

__device__ __forceinline__ f2 add(f2 a, f2 b) {
  f2 d;
  asm("add.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
  return d;
}
__device__ __forceinline__ f2 sub(f2 a, f2 b) {
  f2 d;
  asm("sub.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
  return d;
}
__device__ __forceinline__ f2 mul(f2 a, f2 b) {
  f2 d;
  asm("mul.rn.ftz.f32x2 %0, %1, %2;" : "=l"(d.v) : "l"(a.v), "l"(b.v));
  return d;
}
__device__ __forceinline__ f2 fma(f2 a, f2 b, f2 c) {
  f2 d;
  asm("fma.rn.ftz.f32x2 %0, %1, %2, %3;" : "=l"(d.v) : "l"(a.v), "l"(b.v), "l"(c.v));
  return d;
}
__device__ __forceinline__ f2 rcp(f2 a) {
  float x, y;
  unpack(a, x, y);
  return pack(rcp(x), rcp(y));
}
__device__ __forceinline__ f2 sqrt_(f2 a) {
  float x, y;
  unpack(a, x, y);
  return pack(sqrt_(x), sqrt_(y));
}

// comparisons, selections and predicate logic
__device__ __forceinline__ bool lt(float a, float b) { return a < b; }
__device__ __forceinline__ bool le(float a, float b) { return a <= b; }
__device__ __forceinline__ float sel(bool m, float a, float b) { return m ? a : b; }
__device__ __forceinline__ bool mor(bool a, bool b) { return a || b; }
__device__ __forceinline__ bool mnot(bool a) { return !a; }
__device__ __forceinline__ bool msel(bool c, bool a, bool b) { return c ? a : b; }

__device__ __forceinline__ m2 lt(f2 a, f2 b) {
  float a0, a1, b0, b1;
  unpack(a, a0, a1);
  unpack(b, b0, b1);
  return m2{a0 < b0, a1 < b1};
}
__device__ __forceinline__ m2 le(f2 a, f2 b) {
  float a0, a1, b0, b1;
  unpack(a, a0, a1);
  unpack(b, b0, b1);
  return m2{a0 <= b0, a1 <= b1};
}
__device__ __forceinline__ f2 sel(m2 m, f2 a, f2 b) {
  float a0, a1, b0, b1;
  unpack(a, a0, a1);
  unpack(b, b0, b1);
  return pack(m.x ? a0 : b0, m.y ? a1 : b1);
}
__device__ __forceinline__ m2 mor(m2 a, m2 b) { return m2{a.x || b.x, a.y || b.y}; }
__device__ __forceinline__ m2 mnot(m2 a) { return m2{!a.x, !a.y}; }
__device__ __forceinline__ m2 msel(m2 c, m2 a, m2 b) {
  return m2{c.x ? a.x : b.x, c.y ? a.y : b.y};
}

template <class T> __device__ __forceinline__ T splat(float c);
template <> __device__ __forceinline__ float splat<float>(float c) { return c; }
template <> __device__ __forceinline__ f2 splat<f2>(float c) { return pack(c, c); }

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

// the constants of the algebra in the number type T
template <class T> struct K {
  T g, gm1, gm1inv, qc, omqc, half, quarter, neghalf, one, zero, floor;
};
template <class T> __device__ __forceinline__ K<T> kconsts(const Consts<float> &c) {
  K<T> k;
  k.g = splat<T>(c.g);
  k.gm1 = splat<T>(c.gm1);
  k.gm1inv = splat<T>(c.gm1inv);
  k.qc = splat<T>(c.qc);
  k.omqc = splat<T>(1.0f - c.qc);
  k.half = splat<T>(0.5f);
  k.quarter = splat<T>(0.25f);
  k.neghalf = splat<T>(-0.5f);
  k.one = splat<T>(1.0f);
  k.zero = splat<T>(0.0f);
  k.floor = splat<T>(1e-2f);
  return k;
}

// a state in the frame of a wall: density, velocity across the wall (un)
// and along it (ut), pressure; a flux in the same frame
template <class T> struct NS {
  T rho, un, ut, p;
};
template <class T> struct NF {
  T fd, fn, ft, fe;
};

// minmod of two differences (hs::absmaller's value: the one of smaller
// magnitude when both have the same sign, else zero) in four bit and
// min/max operations: sign(a) max(0, min(|a|, sign(a) b))
__device__ __forceinline__ float minmod(float a, float b) {
  const unsigned sa = __float_as_uint(a) & 0x80000000u;
  const float m = fmaxf(0.0f, fminf(fabsf(a), __uint_as_float(__float_as_uint(b) ^ sa)));
  return __uint_as_float(__float_as_uint(m) | sa);
}
__device__ __forceinline__ f2 minmod(f2 a, f2 b) {
  float a0, a1, b0, b1;
  unpack(a, a0, a1);
  unpack(b, b0, b1);
  return pack(minmod(a0, b0), minmod(a1, b1));
}

// interpolateSingle 2 (hs::muscl) with minmod: face values left (l) and
// right (r) of the wall between x1 and x2
__device__ __forceinline__ void muscl(float x0, float x1, float x2, float x3, float &l, float &r) {
  l = fma(minmod(sub(x1, x0), sub(x2, x1)), 0.5f, x1);
  r = fma(minmod(sub(x2, x1), sub(x3, x2)), -0.5f, x2);
}

// soundSpeed' dens pres = sqrt (gamma * pres / dens)
template <class T> __device__ __forceinline__ T sound(const K<T> &k, T rho, T p) {
  return sqrt_(mul(mul(k.g, p), rcp(rho)));
}

// hllc i left right (HydroMain.hs:237-268) in the frame of the wall
template <class T>
__device__ __forceinline__ NF<T> hllc_ns(const K<T> &k, const NS<T> &L, T cl, const NS<T> &R,
                                         T cr) {
  // densMid * soundMid = (rhoL + rhoR)(cL + cR) / 4
  const T ds = mul(mul(add(L.rho, R.rho), add(cl, cr)), k.quarter);
  const T psraw = fma(ds, sub(L.un, R.un), mul(add(L.p, R.p), k.half));
  const T presStar = sel(lt(k.zero, psraw), psraw, k.zero);
  const T tL = sqrt_(fma(mul(k.qc, rcp(L.p)), presStar, k.omqc));
  const T tR = sqrt_(fma(mul(k.qc, rcp(R.p)), presStar, k.omqc));
  const T qL = sel(le(L.p, presStar), k.one, tL);
  const T qR = sel(le(R.p, presStar), k.one, tR);
  const T cqL = mul(cl, qL), cqR = mul(cr, qR);
  const T shockLeft = sub(L.un, cqL), shockRight = add(R.un, cqR);
  const T mL = mul(L.rho, cqL), mR = mul(R.rho, cqR);
  const T shockStar =
      mul(fma(mR, R.un, fma(mL, L.un, sub(L.p, R.p))), rcp(add(mL, mR)));
  // select (0 < SL) L (select (0 < S*) L* (select (0 < SR) R* R))
  const auto posL = lt(k.zero, shockLeft), posS = lt(k.zero, shockStar),
             posR = lt(k.zero, shockRight);
  const auto useL = mor(posL, posS);
  const auto star = msel(useL, mnot(posL), posR);
  const T r = sel(useL, L.rho, R.rho), p = sel(useL, L.p, R.p);
  const T un = sel(useL, L.un, R.un), ut = sel(useL, L.ut, R.ut);
  const T shock = sel(useL, shockLeft, shockRight);
  const T E = fma(mul(k.half, r), fma(un, un, mul(ut, ut)), mul(k.gm1inv, p));
  const T su = sub(shock, un);
  const T idS = rcp(sub(shock, shockStar));
  const T rsu = mul(r, su);
  const T dens = mul(rsu, idS);
  const T enrg = mul(fma(sub(shockStar, un), fma(rsu, shockStar, p), mul(E, su)), idS);
  const T pst =
      mul(k.gm1, fma(mul(k.neghalf, dens), fma(shockStar, shockStar, mul(ut, ut)), enrg));
  const T fr = sel(star, dens, r), fu = sel(star, shockStar, un);
  const T fE = sel(star, enrg, E), fp = sel(star, pst, p);
  const T mn = mul(fr, fu);
  NF<T> f;
  f.fd = mn;
  f.fn = fma(mn, fu, fp);
  f.ft = mul(mn, ut);
  f.fe = mul(add(fE, fp), fu);
  return f;
}

// the conservative update of hs::update (axis 1 walls, then axis 0 walls,
// then bindPrimitive with the 1e-2 floors), one reciprocal of the density;
// q: the new (rho, v0, v1, p); cons (optional): the conserved state before
// the primitive recovery
template <class T>
__device__ __forceinline__ void update_t(const K<T> &k, T rho, T v0, T v1, T p, T dtdx0,
                                         T dtdx1, const NF<T> &l0, const NF<T> &r0,
                                         const NF<T> &l1, const NF<T> &r1, T *q,
                                         T *cons = nullptr) {
  // fluxes here in axis order: fd, fm0 (in fn), fm1 (in ft), fe
  const T m0 = mul(rho, v0), m1 = mul(rho, v1);
  const T e = fma(k.half, fma(v0, m0, mul(v1, m1)), mul(k.gm1inv, p));
  const T d1 = fma(dtdx1, sub(l1.fd, r1.fd), rho);
  const T a0 = fma(dtdx1, sub(l1.fn, r1.fn), m0);
  const T a1 = fma(dtdx1, sub(l1.ft, r1.ft), m1);
  const T e1 = fma(dtdx1, sub(l1.fe, r1.fe), e);
  const T d2 = fma(dtdx0, sub(l0.fd, r0.fd), d1);
  const T b0 = fma(dtdx0, sub(l0.fn, r0.fn), a0);
  const T b1 = fma(dtdx0, sub(l0.ft, r0.ft), a1);
  const T e2 = fma(dtdx0, sub(l0.fe, r0.fe), e1);
  if (cons) {
    cons[0] = d2;
    cons[1] = b0;
    cons[2] = b1;
    cons[3] = e2;
  }
  const T rd = rcp(d2);
  const T u0 = mul(b0, rd), u1 = mul(b1, rd);
  const T pn = mul(k.gm1, fma(k.neghalf, fma(u0, b0, mul(u1, b1)), e2));
  q[0] = sel(lt(k.floor, d2), d2, k.floor);
  q[1] = u0;
  q[2] = u1;
  q[3] = sel(lt(k.floor, pn), pn, k.floor);
}

// one-wall forms on the axis-ordered records of the tile kernels
template <int AX>
__device__ __forceinline__ Flux<float> hllc(const Consts<float> &c, const Prim<float> &L,
                                            float cl, const Prim<float> &Rt, float cr) {
  const K<float> k = kconsts<float>(c);
  const NS<float> l{L.rho, AX == 0 ? L.v0 : L.v1, AX == 0 ? L.v1 : L.v0, L.p};
  const NS<float> r{Rt.rho, AX == 0 ? Rt.v0 : Rt.v1, AX == 0 ? Rt.v1 : Rt.v0, Rt.p};
  const NF<float> f = hllc_ns<float>(k, l, cl, r, cr);
  Flux<float> o;
  o.fd = f.fd;
  o.fm0 = AX == 0 ? f.fn : f.ft;
  o.fm1 = AX == 0 ? f.ft : f.fn;
  o.fe = f.fe;
  return o;
}

__device__ __forceinline__ NF<float> axis_flux(const Flux<float> &f) {
  return NF<float>{f.fd, f.fm0, f.fm1, f.fe};
}

__device__ __forceinline__ Prim<float> update(const Consts<float> &c, const Prim<float> &b,
                                              float dtdx0, float dtdx1, const Flux<float> &l0,
                                              const Flux<float> &r0, const Flux<float> &l1,
                                              const Flux<float> &r1, float *cons = nullptr) {
  const K<float> k = kconsts<float>(c);
  float q[4];
  update_t<float>(k, b.rho, b.v0, b.v1, b.p, dtdx0, dtdx1, axis_flux(l0), axis_flux(r0),
                  axis_flux(l1), axis_flux(r1), q, cons);
  return Prim<float>{q[0], q[1], q[2], q[3]};
}

__device__ __forceinline__ float sound(const Consts<float> &c, float rho, float p) {
  return sound<float>(kconsts<float>(c), rho, p);
}

}  // namespace hf
}  // namespace om

// om_oracle.cpp -- CPU restatement of the Orthotope Machine kernels that
// Paraiso's generator emits for examples/Life and examples/Hydro.
//
// TEST INFRASTRUCTURE ONLY: the checker for the CUDA library, never part of
// the product path.  Loaded by tests/, __graft_entry__.smoke() and the
// CPU-baseline leg of bench.py.
//
// The arithmetic follows the expression trees of the reference's OM
// builders operation by operation, because the generator prints every
// Arith node as one C operation without constant folding or re-association
// (Language/Paraiso/Generator/PlanTrans.hs:670-710).  Literals are typed
// as the OM's Real (float in the pre-generated sample, double in the current
// examples/Hydro/Hydro.hs:37).  Build with -ffp-contract=off so that no
// multiply-add is fused.
//
// Values that the generated code recomputes at several cursors (Delayed
// nodes, e.g. a wall flux read both as the left wall of one cell and as the
// right wall of its neighbour) are computed once here and stored: the
// expression is the same at every cursor, so the value is the same.

#include "om_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// ---------------------------------------------------------------------------
// synthetic inputs
// ---------------------------------------------------------------------------

static inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

extern "C" uint64_t oracle_hash64(uint64_t seed, uint64_t index) {
  return mix64(mix64(seed) + index * 0x9E3779B97F4A7C15ULL);
}

extern "C" void oracle_hash_uniform_f32(uint64_t seed, size_t n, double lo,
                                        double hi, float *out) {
#pragma omp parallel for schedule(static)
  for (long long i = 0; i < (long long)n; ++i) {
    const double u = (double)(oracle_hash64(seed, (uint64_t)i) >> 11) *
                     (1.0 / 9007199254740992.0);
    out[i] = (float)(lo + (hi - lo) * u);
  }
}

extern "C" void oracle_life_fill_bernoulli(int n0, int n1, int cyclic,
                                           uint64_t seed, double p,
                                           int32_t *cell) {
  const int lm = cyclic ? 0 : 1;
  const int ms0 = n0 + 2 * lm, ms1 = n1 + 2 * lm;
  const uint64_t thr = (uint64_t)std::floor(p * 9007199254740992.0);
  std::memset(cell, 0, sizeof(int32_t) * (size_t)ms0 * ms1);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < n1; ++y)
    for (int x = 0; x < n0; ++x) {
      uint64_t i = (uint64_t)x + (uint64_t)n0 * (uint64_t)y;
      cell[(size_t)(y + lm) * ms0 + (x + lm)] =
          ((oracle_hash64(seed, i) >> 11) < thr) ? 1 : 0;
    }
}

// ---------------------------------------------------------------------------
// Life: examples/Life/Generator.hs:78-115, generated form
// examples-old/Life-exampled/dist/Life.cpp:114-169.
// ---------------------------------------------------------------------------

extern "C" int oracle_life_memory_size(int n, int cyclic) {
  return cyclic ? n : n + 2;
}

extern "C" int32_t oracle_life_step(int n0, int n1, int cyclic,
                                   const int32_t *cur, int32_t *next) {
  const int lm = cyclic ? 0 : 1;
  const int ms0 = n0 + 2 * lm, ms1 = n1 + 2 * lm;
  if (!cyclic) {
    // the manifest's margins are never written by the stencil sub-kernel
    for (int x = 0; x < ms0; ++x) {
      next[x] = 0;
      next[(size_t)(ms1 - 1) * ms0 + x] = 0;
    }
    for (int y = 0; y < ms1; ++y) {
      next[(size_t)y * ms0] = 0;
      next[(size_t)y * ms0 + ms0 - 1] = 0;
    }
  }
  uint32_t pop = 0;
#pragma omp parallel for schedule(static) reduction(+ : pop)
  for (int y = 0; y < n1; ++y) {
    for (int x = 0; x < n0; ++x) {
      // cursor codec: PlanTrans.hs:468-484 (cyclic adds (x+n)%n per axis)
      uint32_t num = 0;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          if (dx == 0 && dy == 0) continue;
          int xx = x + lm + dx, yy = y + lm + dy;
          if (cyclic) {
            xx = (xx + ms0) % ms0;
            yy = (yy + ms1) % ms1;
          }
          num += (uint32_t)cur[(size_t)yy * ms0 + xx];
        }
      const int32_t c = cur[(size_t)(y + lm) * ms0 + (x + lm)];
      const int32_t n = (int32_t)num;
      const bool alive = (c == 0 && n == 3) || (c == 1 && n >= 2 && n <= 3);
      const int32_t v = alive ? 1 : 0;
      next[(size_t)(y + lm) * ms0 + (x + lm)] = v;
      pop += (uint32_t)v;
    }
  }
  return (int32_t)pop;
}

extern "C" void oracle_life_run(int n0, int n1, int cyclic, int steps,
                                int32_t *cell, int32_t *populations) {
  const int lm = cyclic ? 0 : 1;
  const size_t mem = (size_t)(n0 + 2 * lm) * (n1 + 2 * lm);
  std::vector<int32_t> tmp(mem);
  for (int t = 0; t < steps; ++t) {
    int32_t pop = oracle_life_step(n0, n1, cyclic, cell, tmp.data());
    std::memcpy(cell, tmp.data(), mem * sizeof(int32_t));
    if (populations) populations[t] = pop;
  }
}

// ---------------------------------------------------------------------------
// Hydro
// ---------------------------------------------------------------------------

namespace {

// Dual number for the tangent-linear run: value and one directional
// derivative.  Comparisons and selections act on the value, so the
// derivative follows the branch the primal takes.
struct Dual {
  double v, d;
  Dual() : v(0), d(0) {}
  Dual(double x) : v(x), d(0) {}
  Dual(double x, double dx) : v(x), d(dx) {}
};
inline Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
inline Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
inline Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
inline Dual operator*(Dual a, Dual b) {
  return Dual(a.v * b.v, a.d * b.v + a.v * b.d);
}
inline Dual operator/(Dual a, Dual b) {
  double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline Dual dsqrt(Dual a) {
  double s = std::sqrt(a.v);
  return Dual(s, a.d / (2.0 * s));
}
inline double dsqrt(double a) { return std::sqrt(a); }
inline float dsqrt(float a) { return std::sqrt(a); }
inline Dual dabs(Dual a) { return a.v < 0 ? -a : a; }
inline double dabs(double a) { return std::fabs(a); }
inline float dabs(float a) { return std::fabs(a); }
inline double val(Dual a) { return a.v; }
inline double val(double a) { return a; }
inline double val(float a) { return a; }

// Operation-counting number: a double that tallies every arithmetic
// operation the Hydro step performs on it, so the restatement itself gives
// the scheme's floating-point work per cell-update.  Counters are global;
// oracle_hydro_count_ops runs the step on one thread.
enum { kOpAdd, kOpMul, kOpDiv, kOpSqrt, kOpCmp, kOpAbsNeg, kOpKinds };
static long long g_ops[kOpKinds];
struct Counted {
  double v;
  Counted() : v(0) {}
  Counted(double x) : v(x) {}
};
inline Counted operator+(Counted a, Counted b) { ++g_ops[kOpAdd]; return Counted(a.v + b.v); }
inline Counted operator-(Counted a, Counted b) { ++g_ops[kOpAdd]; return Counted(a.v - b.v); }
inline Counted operator-(Counted a) { ++g_ops[kOpAbsNeg]; return Counted(-a.v); }
inline Counted operator*(Counted a, Counted b) { ++g_ops[kOpMul]; return Counted(a.v * b.v); }
inline Counted operator/(Counted a, Counted b) { ++g_ops[kOpDiv]; return Counted(a.v / b.v); }
inline bool operator<(Counted a, Counted b) { ++g_ops[kOpCmp]; return a.v < b.v; }
inline bool operator<=(Counted a, Counted b) { ++g_ops[kOpCmp]; return a.v <= b.v; }
inline bool operator>(Counted a, Counted b) { ++g_ops[kOpCmp]; return a.v > b.v; }
inline Counted dsqrt(Counted a) { ++g_ops[kOpSqrt]; return Counted(std::sqrt(a.v)); }
inline Counted dabs(Counted a) { ++g_ops[kOpAbsNeg]; return Counted(std::fabs(a.v)); }
inline double val(Counted a) { return a.v; }

// std::max / std::min as the generated C++ calls them (PlanTrans.hs:692-693)
template <class R> inline R omax(R a, R b) { return (a < b) ? b : a; }
template <class R> inline R omin(R a, R b) { return (b < a) ? b : a; }

// Primitive-variable record and the derived fields Hydrable computes
// (examples/Hydro/Hydro.hs:99-127).
template <class R> struct Prim {
  R rho, v0, v1, p;
};

template <class R> struct Flux {
  R fd, fm0, fm1, fe;  // density, momentum (component 0,1), energy flux
};

template <class R> struct Ctx {
  R gamma;
};

// kineticEnergy x = 0.5 * contract (\i -> velocity x !i * momentum x !i)
template <class R> inline R kinetic(R v0, R v1, R m0, R m1) {
  return R(0.5) * ((R(0) + v0 * m0) + v1 * m1);
}

// Fluxes along axis `ax` of a record given by primitives
// (bindPrimitive: momentum = rho*v, energy = Ek + 1/(g-1)*p).
template <class R>
inline Flux<R> flux_of_prim(const Ctx<R> &c, int ax, R rho, R v0, R v1, R p) {
  R m0 = rho * v0, m1 = rho * v1;
  R ek = kinetic(v0, v1, m0, m1);
  R e = ek + (R(1) / (c.gamma - R(1))) * p;
  R h = e + p;
  R va = ax == 0 ? v0 : v1;
  Flux<R> f;
  f.fd = ax == 0 ? m0 : m1;
  f.fm0 = m0 * va + p * (ax == 0 ? R(1) : R(0));
  f.fm1 = m1 * va + p * (ax == 1 ? R(1) : R(0));
  f.fe = h * va;
  return f;
}

// Fluxes along `ax` of a record given by conserved variables
// (bindConserved: velocity = m/rho, pressure = (g-1)*(E - Ek)).
template <class R>
inline Flux<R> flux_of_cons(const Ctx<R> &c, int ax, R rho, R m0, R m1, R e) {
  R v0 = m0 / rho, v1 = m1 / rho;
  R ek = kinetic(v0, v1, m0, m1);
  R p = (c.gamma - R(1)) * (e - ek);
  R h = e + p;
  R va = ax == 0 ? v0 : v1;
  Flux<R> f;
  f.fd = ax == 0 ? m0 : m1;
  f.fm0 = m0 * va + p * (ax == 0 ? R(1) : R(0));
  f.fm1 = m1 * va + p * (ax == 1 ? R(1) : R(0));
  f.fe = h * va;
  return f;
}

// soundSpeed' dens pres = sqrt (kGamma * pres / dens)   (Hydro.hs:57-58)
template <class R> inline R sound(const Ctx<R> &c, R rho, R p) {
  return dsqrt((c.gamma * p) / rho);
}

// hllcQ sp p (HydroMain.hs:270-271), condition kept as written
template <class R> inline R hllc_q(const Ctx<R> &c, R sp, R p) {
  R t = dsqrt(R(1) + (c.gamma + R(1)) / (R(2) * c.gamma) * (sp / p - R(1)));
  return (p <= sp) ? R(1) : t;
}

// starState (HydroMain.hs:272-282): conserved star state, then its flux
template <class R>
inline Flux<R> star_flux(const Ctx<R> &c, int ax, R sstar, R shock, R rho,
                         R v0, R v1, R p) {
  R speed = ax == 0 ? v0 : v1;
  R dens = rho * (shock - speed) / (shock - sstar);
  R mome0 = dens * (ax == 0 ? sstar : v0);
  R mome1 = dens * (ax == 1 ? sstar : v1);
  R m0 = rho * v0, m1 = rho * v1;
  R ek = kinetic(v0, v1, m0, m1);
  R e = ek + (R(1) / (c.gamma - R(1))) * p;
  R enrg = dens * (e / rho + (sstar - speed) * (sstar + p / rho / (shock - speed)));
  return flux_of_cons(c, ax, dens, mome0, mome1, enrg);
}

// hllc i left right (HydroMain.hs:237-268): the wall record's fluxes
template <class R>
inline Flux<R> hllc(const Ctx<R> &c, int ax, const Prim<R> &L,
                    const Prim<R> &Rt) {
  R cl = sound(c, L.rho, L.p), cr = sound(c, Rt.rho, Rt.p);
  R densMid = (L.rho + Rt.rho) / R(2);
  R soundMid = (cl + cr) / R(2);
  R uL = ax == 0 ? L.v0 : L.v1;
  R uR = ax == 0 ? Rt.v0 : Rt.v1;
  R presStar = omax(R(0), (L.p + Rt.p) / R(2) - densMid * soundMid * (uR - uL));
  R shockLeft = uL - cl * hllc_q(c, presStar, L.p);
  R shockRight = uR + cr * hllc_q(c, presStar, Rt.p);
  R shockStar = (Rt.p - L.p + L.rho * uL * (shockLeft - uL) -
                 Rt.rho * uR * (shockRight - uR)) /
                (L.rho * (shockLeft - uL) - Rt.rho * (shockRight - uR));
  if (R(0) < shockLeft) return flux_of_prim(c, ax, L.rho, L.v0, L.v1, L.p);
  if (R(0) < shockStar)
    return star_flux(c, ax, shockStar, shockLeft, L.rho, L.v0, L.v1, L.p);
  if (R(0) < shockRight)
    return star_flux(c, ax, shockStar, shockRight, Rt.rho, Rt.v0, Rt.v1, Rt.p);
  return flux_of_prim(c, ax, Rt.rho, Rt.v0, Rt.v1, Rt.p);
}

// absmaller a b (HydroMain.hs:227)
template <class R> inline R absmaller(R a, R b) {
  return (a * b <= R(0)) ? R(0) : ((dabs(a) < dabs(b)) ? a : b);
}

// interpolateSingle 2 (HydroMain.hs:219-231): (left, right) face values
template <class R>
inline void muscl(R x0, R x1, R x2, R x3, R &l, R &r) {
  R d01 = x1 - x0, d12 = x2 - x1, d23 = x3 - x2;
  R d1 = absmaller(d01, d12);
  R d2 = absmaller(d12, d23);
  l = x1 + d1 / R(2);
  r = x2 - d2 / R(2);
}

template <class R> struct Grid {
  int n0, n1, cyclic, lm, ms0, ms1;
  size_t mem;
  size_t at(int x, int y) const {  // memory coordinates, wrapped if cyclic
    if (cyclic) {
      x = (x % ms0 + ms0) % ms0;
      y = (y % ms1 + ms1) % ms1;
    }
    return (size_t)y * ms0 + x;
  }
};

template <class R> struct State {
  std::vector<R> rho, v0, v1, p;
  explicit State(size_t n) : rho(n), v0(n), v1(n), p(n) {}
  Prim<R> get(size_t i) const { return Prim<R>{rho[i], v0[i], v1[i], p[i]}; }
  void set(size_t i, const Prim<R> &q) {
    rho[i] = q.rho; v0[i] = q.v0; v1[i] = q.v1; p[i] = q.p;
  }
};

// Jet state of boundaryCondition / buildInit (HydroMain.hs:79-131).
template <class R>
inline void jet_region(const Ctx<R> &c, R dR0, R dR1, R ext1, int ix, int iy,
                       bool &region) {
  R cx = dR0 * R(ix), cy = dR1 * R(iy);
  region = (cy > R(0.47) * ext1) && ((cy < R(0.53) * ext1) && (cx < R(0)));
  (void)c;
}

template <class R>
inline Prim<R> jet_state(const Ctx<R> &c, bool region) {
  Prim<R> q;
  q.rho = c.gamma * c.gamma * (region ? R(1) : R(10));
  q.v0 = region ? R(6) : R(0);
  q.v1 = region ? R(0) : R(0);
  q.p = R(0.6);
  return q;
}

// One conservative update of base cell `b` by the two axes' walls:
// cellN = addFlux ax0 (addFlux ax1 cellS)   (HydroMain.hs:171-196),
// then bindPrimitive (max 1e-2 rho) v (max 1e-2 p).
template <class R>
inline Prim<R> update(const Ctx<R> &c, const Prim<R> &b, R dtdx0, R dtdx1,
                      const Flux<R> &l0, const Flux<R> &r0, const Flux<R> &l1,
                      const Flux<R> &r1) {
  R m0 = b.rho * b.v0, m1 = b.rho * b.v1;
  R ek = kinetic(b.v0, b.v1, m0, m1);
  R e = ek + (R(1) / (c.gamma - R(1))) * b.p;
  // axis 1 first
  R d1 = b.rho + dtdx1 * (l1.fd - r1.fd);
  R a0 = m0 + dtdx1 * (l1.fm0 - r1.fm0);
  R a1 = m1 + dtdx1 * (l1.fm1 - r1.fm1);
  R e1 = e + dtdx1 * (l1.fe - r1.fe);
  // then axis 0
  R d2 = d1 + dtdx0 * (l0.fd - r0.fd);
  R b0 = a0 + dtdx0 * (l0.fm0 - r0.fm0);
  R b1 = a1 + dtdx0 * (l0.fm1 - r0.fm1);
  R e2 = e1 + dtdx0 * (l0.fe - r0.fe);
  R v0 = b0 / d2, v1 = b1 / d2;
  R ekn = kinetic(v0, v1, b0, b1);
  R pn = (c.gamma - R(1)) * (e2 - ekn);
  Prim<R> q;
  q.rho = omax(R(1e-2), d2);
  q.v0 = v0;
  q.v1 = v1;
  q.p = omax(R(1e-2), pn);
  return q;
}

template <class R>
R hydro_step(const oracle_hydro_shape &s, R cfl, R dR0, R dR1, R ext0, R ext1,
             R *time, R *dens, R *vx, R *vy, R *pres) {
  (void)ext0;
  Ctx<R> c{R(s.gamma)};
  Grid<R> g;
  g.n0 = s.n0; g.n1 = s.n1; g.cyclic = s.cyclic;
  g.lm = s.cyclic ? 0 : 3;
  g.ms0 = s.n0 + 2 * g.lm; g.ms1 = s.n1 + 2 * g.lm;
  g.mem = (size_t)g.ms0 * g.ms1;
  const int ms0 = g.ms0, ms1 = g.ms1, lm = g.lm;

  // boundaryCondition: cells whose index is outside [0,n) take the jet state
  State<R> P(g.mem);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < ms1; ++y)
    for (int x = 0; x < ms0; ++x) {
      size_t i = (size_t)y * ms0 + x;
      Prim<R> q{dens[i], vx[i], vy[i], pres[i]};
      if (!s.cyclic) {
        int ix = x - lm, iy = y - lm;
        bool outOf = (ix < 0 || iy < 0) || (ix >= s.n0 || iy >= s.n1);
        if (outOf) {
          bool region;
          jet_region(c, dR0, dR1, ext1, ix, iy, region);
          q = jet_state(c, region);
        }
      }
      P.set(i, q);
    }

  // timescale and reduce Min over the whole memory array (HydroMain.hs:150-154)
  R dtmin = R(0);
  {
    std::vector<R> ts(g.mem);
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < g.mem; ++i) {
      R cs = sound(c, P.rho[i], P.p[i]);
      R t0 = dR0 / (cs + dabs(P.v0[i]));
      R t1 = dR1 / (cs + dabs(P.v1[i]));
      ts[i] = omin(t0, t1);
    }
    dtmin = ts[0];
    for (size_t i = 1; i < g.mem; ++i) dtmin = omin(dtmin, ts[i]);
  }
  const R dtG = cfl * dtmin;
  const R dtHalf = dtG / R(2);

  // x-range / y-range of cells computed in each stage (memory coordinates)
  const int s1lo0 = s.cyclic ? 0 : 1, s1hi0 = s.cyclic ? ms0 : ms0 - 1;
  const int s1lo1 = s.cyclic ? 0 : 1, s1hi1 = s.cyclic ? ms1 : ms1 - 1;

  // stage 1: order-1 walls on P, update of P by dt/2
  State<R> C2(g.mem);
  {
    std::vector<Flux<R>> w0(g.mem), w1(g.mem);
#pragma omp parallel for schedule(static)
    for (int y = s1lo1; y < s1hi1; ++y)
      for (int x = s1lo0; x < s1hi0 + (s.cyclic ? 0 : 1); ++x) {
        if (x >= ms0) continue;
        w0[(size_t)y * ms0 + x] = hllc(c, 0, P.get(g.at(x - 1, y)), P.get(g.at(x, y)));
      }
#pragma omp parallel for schedule(static)
    for (int y = s1lo1; y < s1hi1 + (s.cyclic ? 0 : 1); ++y)
      for (int x = s1lo0; x < s1hi0; ++x) {
        if (y >= ms1) continue;
        w1[(size_t)y * ms0 + x] = hllc(c, 1, P.get(g.at(x, y - 1)), P.get(g.at(x, y)));
      }
    const R dtdx0 = dtHalf / dR0, dtdx1 = dtHalf / dR1;
#pragma omp parallel for schedule(static)
    for (int y = s1lo1; y < s1hi1; ++y)
      for (int x = s1lo0; x < s1hi0; ++x) {
        size_t i = (size_t)y * ms0 + x;
        C2.set(i, update(c, P.get(i), dtdx0, dtdx1, w0[i], w0[g.at(x + 1, y)],
                         w1[i], w1[g.at(x, y + 1)]));
      }
  }

  // stage 2: order-2 walls on C2, update of P by dt
  {
    const int lo0 = s.cyclic ? 0 : lm, hi0 = s.cyclic ? ms0 : ms0 - lm;
    const int lo1 = s.cyclic ? 0 : lm, hi1 = s.cyclic ? ms1 : ms1 - lm;
    std::vector<Flux<R>> w0(g.mem), w1(g.mem);
#pragma omp parallel for schedule(static)
    for (int y = lo1; y < hi1; ++y)
      for (int x = lo0; x < hi0 + (s.cyclic ? 0 : 1); ++x) {
        Prim<R> a0 = C2.get(g.at(x - 2, y)), a1 = C2.get(g.at(x - 1, y));
        Prim<R> a2 = C2.get(g.at(x, y)), a3 = C2.get(g.at(x + 1, y));
        Prim<R> L, Rt;
        muscl(a0.rho, a1.rho, a2.rho, a3.rho, L.rho, Rt.rho);
        muscl(a0.v0, a1.v0, a2.v0, a3.v0, L.v0, Rt.v0);
        muscl(a0.v1, a1.v1, a2.v1, a3.v1, L.v1, Rt.v1);
        muscl(a0.p, a1.p, a2.p, a3.p, L.p, Rt.p);
        w0[g.at(x, y)] = hllc(c, 0, L, Rt);
      }
#pragma omp parallel for schedule(static)
    for (int y = lo1; y < hi1 + (s.cyclic ? 0 : 1); ++y)
      for (int x = lo0; x < hi0; ++x) {
        Prim<R> a0 = C2.get(g.at(x, y - 2)), a1 = C2.get(g.at(x, y - 1));
        Prim<R> a2 = C2.get(g.at(x, y)), a3 = C2.get(g.at(x, y + 1));
        Prim<R> L, Rt;
        muscl(a0.rho, a1.rho, a2.rho, a3.rho, L.rho, Rt.rho);
        muscl(a0.v0, a1.v0, a2.v0, a3.v0, L.v0, Rt.v0);
        muscl(a0.v1, a1.v1, a2.v1, a3.v1, L.v1, Rt.v1);
        muscl(a0.p, a1.p, a2.p, a3.p, L.p, Rt.p);
        w1[g.at(x, y)] = hllc(c, 1, L, Rt);
      }
    const R dtdx0 = dtG / dR0, dtdx1 = dtG / dR1;
    // the output manifests are zero outside the stage-2 region
    if (!s.cyclic) {
      std::fill(dens, dens + g.mem, R(0));
      std::fill(vx, vx + g.mem, R(0));
      std::fill(vy, vy + g.mem, R(0));
      std::fill(pres, pres + g.mem, R(0));
    }
#pragma omp parallel for schedule(static)
    for (int y = lo1; y < hi1; ++y)
      for (int x = lo0; x < hi0; ++x) {
        size_t i = (size_t)y * ms0 + x;
        Prim<R> q = update(c, P.get(i), dtdx0, dtdx1, w0[i], w0[g.at(x + 1, y)],
                           w1[i], w1[g.at(x, y + 1)]);
        dens[i] = q.rho; vx[i] = q.v0; vy[i] = q.v1; pres[i] = q.p;
      }
  }
  *time = *time + dtG;
  return dtG;
}

template <class R>
void init_jet(const oracle_hydro_shape &s, R dR0, R dR1, R ext0, R ext1,
              R *dens, R *vx, R *vy, R *pres) {
  (void)ext0;
  Ctx<R> c{R(s.gamma)};
  const int lm = s.cyclic ? 0 : 3;
  const int ms0 = s.n0 + 2 * lm, ms1 = s.n1 + 2 * lm;
  const R pi = R(3.141592653589793);
#pragma omp parallel for schedule(static)
  for (int y = 0; y < ms1; ++y)
    for (int x = 0; x < ms0; ++x) {
      size_t i = (size_t)y * ms0 + x;
      const int ix = x - lm, iy = y - lm;
      R cx = dR0 * R(ix), cy = dR1 * R(iy);
      bool region = (cy > R(0.47) * ext1) && ((cy < R(0.53) * ext1) && (cx < R(0)));
      R factor = R(1) + R(1e-3) * R(std::sin(val(R(6) * pi * cx)));
      dens[i] = factor * c.gamma * c.gamma * (region ? R(1) : R(10));
      vx[i] = region ? R(6) : R(0);
      vy[i] = region ? R(0) : R(0);
      pres[i] = factor * R(0.6);
    }
}

template <class R>
void init_kh(int n0, int n1, uint64_t seed, R *dens, R *vx, R *vy, R *pres) {
  const double pi = 3.141592653589793;
#pragma omp parallel for schedule(static)
  for (int y = 0; y < n1; ++y)
    for (int x = 0; x < n0; ++x) {
      const size_t i = (size_t)y * n0 + x;
      const double cx = (x + 0.5) / n0, cy = (y + 0.5) / n1;
      const bool band = std::fabs(cy - 0.5) < 0.25;
      const double u = (double)(oracle_hash64(seed, i) >> 11) * (1.0 / 9007199254740992.0);
      dens[i] = (R)(band ? 2.0 : 1.0);
      vx[i] = (R)(band ? 0.5 : -0.5);
      vy[i] = (R)(0.01 * std::sin(4.0 * pi * cx) + 0.01 * (2.0 * u - 1.0));
      pres[i] = (R)2.5;
    }
}

struct Neumaier {
  double s = 0, c = 0;
  void add(double x) {
    double t = s + x;
    if (std::fabs(s) >= std::fabs(x)) c += (s - t) + x;
    else c += (x - t) + s;
    s = t;
  }
  double get() const { return s + c; }
};

template <class R>
void totals(const oracle_hydro_shape &s, const R *dens, const R *vx,
            const R *vy, const R *pres, double *out) {
  const int lm = s.cyclic ? 0 : 3;
  const int ms0 = s.n0 + 2 * lm;
  const double g = s.gamma;
  Neumaier a, b, cc, d;
  for (int y = 0; y < s.n1; ++y)
    for (int x = 0; x < s.n0; ++x) {
      size_t i = (size_t)(y + lm) * ms0 + (x + lm);
      double r = dens[i], u = vx[i], v = vy[i], p = pres[i];
      a.add(r);
      b.add(r * u);
      cc.add(r * v);
      d.add(0.5 * r * (u * u + v * v) + p / (g - 1.0));
    }
  out[0] = a.get(); out[1] = b.get(); out[2] = cc.get(); out[3] = d.get();
}

}  // namespace

extern "C" int oracle_hydro_memory_size(int n, int cyclic) {
  return cyclic ? n : n + 6;
}

extern "C" double oracle_hydro_step_f64(oracle_hydro_shape s, double cfl,
                                        double dR0, double dR1, double extent0,
                                        double extent1, double *time,
                                        double *dens, double *vx, double *vy,
                                        double *pres) {
  return hydro_step<double>(s, cfl, dR0, dR1, extent0, extent1, time, dens, vx,
                            vy, pres);
}

extern "C" float oracle_hydro_step_f32(oracle_hydro_shape s, float cfl,
                                       float dR0, float dR1, float extent0,
                                       float extent1, float *time, float *dens,
                                       float *vx, float *vy, float *pres) {
  return hydro_step<float>(s, cfl, dR0, dR1, extent0, extent1, time, dens, vx,
                           vy, pres);
}

extern "C" void oracle_hydro_init_jet_f64(oracle_hydro_shape s, double dR0,
                                          double dR1, double extent0,
                                          double extent1, double *dens,
                                          double *vx, double *vy,
                                          double *pres) {
  init_jet<double>(s, dR0, dR1, extent0, extent1, dens, vx, vy, pres);
}

extern "C" void oracle_hydro_init_jet_f32(oracle_hydro_shape s, float dR0,
                                          float dR1, float extent0,
                                          float extent1, float *dens,
                                          float *vx, float *vy, float *pres) {
  init_jet<float>(s, dR0, dR1, extent0, extent1, dens, vx, vy, pres);
}

extern "C" void oracle_hydro_init_kh_f64(int n0, int n1, uint64_t seed,
                                         double *dens, double *vx, double *vy,
                                         double *pres) {
  init_kh<double>(n0, n1, seed, dens, vx, vy, pres);
}

extern "C" void oracle_hydro_init_kh_f32(int n0, int n1, uint64_t seed,
                                         float *dens, float *vx, float *vy,
                                         float *pres) {
  init_kh<float>(n0, n1, seed, dens, vx, vy, pres);
}

extern "C" void oracle_hydro_totals_f64(oracle_hydro_shape s,
                                        const double *dens, const double *vx,
                                        const double *vy, const double *pres,
                                        double *out) {
  totals<double>(s, dens, vx, vy, pres, out);
}

extern "C" void oracle_hydro_totals_f32(oracle_hydro_shape s,
                                        const float *dens, const float *vx,
                                        const float *vy, const float *pres,
                                        double *out) {
  totals<float>(s, dens, vx, vy, pres, out);
}

extern "C" double oracle_hydro_step_tl_f64(oracle_hydro_shape s, double cfl,
                                           double dR0, double dR1, double *time,
                                           double *dens, double *vx,
                                           double *vy, double *pres,
                                           double *d_dens, double *d_vx,
                                           double *d_vy, double *d_pres) {
  const int lm = s.cyclic ? 0 : 3;
  const size_t mem = (size_t)(s.n0 + 2 * lm) * (s.n1 + 2 * lm);
  std::vector<Dual> r(mem), u(mem), v(mem), p(mem);
  for (size_t i = 0; i < mem; ++i) {
    r[i] = Dual(dens[i], d_dens[i]);
    u[i] = Dual(vx[i], d_vx[i]);
    v[i] = Dual(vy[i], d_vy[i]);
    p[i] = Dual(pres[i], d_pres[i]);
  }
  Dual t(*time);
  Dual dt = hydro_step<Dual>(s, Dual(cfl), Dual(dR0), Dual(dR1), Dual(1.0),
                             Dual(1.0), &t, r.data(), u.data(), v.data(),
                             p.data());
  for (size_t i = 0; i < mem; ++i) {
    dens[i] = r[i].v; d_dens[i] = r[i].d;
    vx[i] = u[i].v; d_vx[i] = u[i].d;
    vy[i] = v[i].v; d_vy[i] = v[i].d;
    pres[i] = p[i].v; d_pres[i] = p[i].d;
  }
  *time = t.v;
  return dt.v;
}

/* Floating-point operations of one Hydro step of the n0 x n1 periodic
 * Kelvin-Helmholtz start (seed), counted on the restatement (one thread):
 * out = {add/sub, mul, div, sqrt, compare, abs/neg} over the whole step. */
extern "C" void oracle_hydro_count_ops(int n0, int n1, uint64_t seed, double gamma,
                                       double cfl, long long *out) {
  const size_t mem = (size_t)n0 * n1;
  std::vector<double> r(mem), u(mem), v(mem), p(mem);
  init_kh<double>(n0, n1, seed, r.data(), u.data(), v.data(), p.data());
  std::vector<Counted> cr(r.begin(), r.end()), cu(u.begin(), u.end()), cv(v.begin(), v.end()),
      cp(p.begin(), p.end());
  oracle_hydro_shape s;
  s.n0 = n0; s.n1 = n1; s.cyclic = 1; s.gamma = gamma;
  Counted t(0.0);
#ifdef _OPENMP
  const int threads = omp_get_max_threads();
  omp_set_num_threads(1);
#endif
  for (int k = 0; k < kOpKinds; ++k) g_ops[k] = 0;
  hydro_step<Counted>(s, Counted(cfl), Counted(1.0 / n0), Counted(1.0 / n1), Counted(1.0),
                      Counted(1.0), &t, cr.data(), cu.data(), cv.data(), cp.data());
  for (int k = 0; k < kOpKinds; ++k) out[k] = g_ops[k];
#ifdef _OPENMP
  omp_set_num_threads(threads);
#endif
}

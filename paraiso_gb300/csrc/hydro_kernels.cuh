// hydro_kernels.cuh -- Hydro step kernels, templated on the real type.
// Included by hydro_exact.cu (no multiply-add contraction: bit-exact with
// the generated code's arithmetic) and hydro_fast.cu (contraction allowed).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "hydro_scheme.cuh"

namespace om {

// Device scalar block of a Hydro handle.  The first fields are the OM's
// statics (HydroMain.hs:44-53); the rest are runtime state.
struct HydroScalars {
  int32_t generation;
  int32_t pad0;
  double time, cfl, dR0, dR1, extent0, extent1;
  // bit pattern of the CFL minimum of the current state (see hk::ts_bits),
  // double-buffered by step parity
  unsigned long long tsmin[2];
  double dt_last;
  // cfl, dR0, dR1 and extent1 rounded to float by the host whenever it
  // uploads the block (hydro_scalars_refresh), so that FP32 kernels need no
  // per-thread conversion from double; (float)x is the same rounding either
  // side
  float cfl_f, dR0_f, dR1_f, ext1_f;
  // raised by a kernel whose bounded wait for its tensor copies ran out
  uint32_t wait_error;
};

// the float copies of a scalar block (host side, before every upload)
inline void hydro_scalars_refresh(HydroScalars *s) {
  s->cfl_f = (float)s->cfl;
  s->dR0_f = (float)s->dR0;
  s->dR1_f = (float)s->dR1;
  s->ext1_f = (float)s->extent1;
}

struct HydroStepArgs {
  const void *rho, *v0, *v1, *p;   // current state (memory-sized arrays)
  void *nrho, *nv0, *nv1, *np;     // next state
  int n0, n1;                      // grid (cyclic, no margins)
  int nt0;                         // tiles along x
  double gamma;
  float gamma_f;                   // (float)gamma
  HydroScalars *sc;
  int read_slot;                   // tsmin slot holding min of the current state
  double *dt_hist;                 // dt of this step is written to dt_hist[0]
  // open boundary only (the OPEN kernels): margin width, memory row pitch
  // (n0 + 2 lm) and the CFL timescale minimum of the margin cells
  int lm, ms0;
  const unsigned long long *margin_min;
  // persistent kernels: at most this many CTAs (0 = as many as stay
  // resident); read by the host launcher only
  int grid_limit;
};

// What a taped step keeps for the reverse sweep (periodic grids; arrays of
// n0 x n1 values of the OM's Real type): the stage-1 state q; per stage the
// flux differences (left wall - right wall) of each axis that the
// conservative update adds, d[4 * axis + k] for k = density, momentum 0,
// momentum 1, energy; and the stage-2 conserved state before the primitive
// recovery, u2 (density, momentum 0, momentum 1, energy).
struct HydroTapeOut {
  void *q[4];
  void *d1[8];
  void *d2[8];
  void *u2[4];
};

namespace hk {

// A CFL minimum is kept as the bit pattern of a positive value of the OM's
// Real type (float bits zero-extended, or double bits): the bit patterns of
// positive IEEE values order like the values, so atomicMin on them is a min.
template <class R> __device__ __forceinline__ unsigned long long ts_bits(R t);
template <> __device__ __forceinline__ unsigned long long ts_bits<float>(float t) {
  return (unsigned long long)__float_as_uint(t);
}
template <> __device__ __forceinline__ unsigned long long ts_bits<double>(double t) {
  return (unsigned long long)__double_as_longlong(t);
}

template <class R> __device__ __forceinline__ R ts_from_bits(unsigned long long b);
template <> __device__ __forceinline__ float ts_from_bits<float>(unsigned long long b) {
  return __uint_as_float((unsigned int)b);
}
template <> __device__ __forceinline__ double ts_from_bits<double>(unsigned long long b) {
  return __longlong_as_double((long long)b);
}

// block-wide min of CFL bit patterns folded into *dst
__device__ __forceinline__ void block_min_to(unsigned long long v, unsigned long long *dst,
                                             unsigned long long *red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    v = lane < nw ? red[lane] : ~0ull;
    for (int o = 16; o > 0; o >>= 1) {
      unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
      v = w < v ? w : v;
    }
    if (lane == 0) atomicMin(dst, v);
  }
}

template <class R>
__device__ __forceinline__ int wrap(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// periodic index for -n <= i < 2n (one add or subtract, no division)
__device__ __forceinline__ int wrap_near(int i, int n) {
  return i < 0 ? i + n : (i >= n ? i - n : i);
}

// boundaryCondition (HydroMain.hs:105-131): a cell of an open grid whose
// index (ix, iy) lies outside [0, n) holds the jet state, in the OM's Real
// type and operation order
template <class R>
__device__ __forceinline__ hs::Prim<R> jet_state(R g, R dR0, R dR1, R ext1, int ix, int iy) {
  const R cx = dR0 * R(ix), cy = dR1 * R(iy);
  const bool region = (cy > R(0.47) * ext1) && ((cy < R(0.53) * ext1) && (cx < R(0)));
  hs::Prim<R> q;
  q.rho = g * g * (region ? R(1) : R(10));
  q.v0 = region ? R(6) : R(0);
  q.v1 = R(0);
  q.p = R(0.6);
  return q;
}

// the flux differences of one cell's update, as hs::update forms them
template <class R>
__device__ __forceinline__ void tape_diffs(void *const *d, size_t gi, const hs::Flux<R> &l0,
                                           const hs::Flux<R> &r0, const hs::Flux<R> &l1,
                                           const hs::Flux<R> &r1) {
  ((R *)d[0])[gi] = l0.fd - r0.fd;
  ((R *)d[1])[gi] = l0.fm0 - r0.fm0;
  ((R *)d[2])[gi] = l0.fm1 - r0.fm1;
  ((R *)d[3])[gi] = l0.fe - r0.fe;
  ((R *)d[4])[gi] = l1.fd - r1.fd;
  ((R *)d[5])[gi] = l1.fm0 - r1.fm0;
  ((R *)d[6])[gi] = l1.fm1 - r1.fm1;
  ((R *)d[7])[gi] = l1.fe - r1.fe;
}

// Scalars in the OM's Real type: the block's float copies for FP32, the
// doubles themselves for FP64 (the same values (R)x would give).
template <class R> struct Reals;
template <> struct Reals<float> {
  static __device__ __forceinline__ float cfl(const HydroScalars *s) { return s->cfl_f; }
  static __device__ __forceinline__ float dR0(const HydroScalars *s) { return s->dR0_f; }
  static __device__ __forceinline__ float dR1(const HydroScalars *s) { return s->dR1_f; }
  static __device__ __forceinline__ float ext1(const HydroScalars *s) { return s->ext1_f; }
  static __device__ __forceinline__ float gamma(const HydroStepArgs &a) { return a.gamma_f; }
};
template <> struct Reals<double> {
  static __device__ __forceinline__ double cfl(const HydroScalars *s) { return s->cfl; }
  static __device__ __forceinline__ double dR0(const HydroScalars *s) { return s->dR0; }
  static __device__ __forceinline__ double dR1(const HydroScalars *s) { return s->dR1; }
  static __device__ __forceinline__ double ext1(const HydroScalars *s) { return s->extent1; }
  static __device__ __forceinline__ double gamma(const HydroStepArgs &a) { return a.gamma; }
};

// dt of this step in the OM's Real type: dtG = cfl * reduce Min dts
template <class R> __device__ __forceinline__ R step_dt(const HydroStepArgs &a) {
  const R tsmin = ts_from_bits<R>(a.sc->tsmin[a.read_slot]);
  return Reals<R>::cfl(a.sc) * tsmin;
}

// 4- or 8-byte asynchronous copy global -> shared, and its group fences
template <class R> __device__ __forceinline__ void cp_async(R *dst, const R *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if (sizeof(R) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// the scheme's wall flux and update in the exact (generated order) or the
// production algebra
template <bool FA, int AX, class R>
__device__ __forceinline__ hs::Flux<R> wall_flux(R g, const hf::Consts<R> &k,
                                                 const hs::Prim<R> &L, R cl,
                                                 const hs::Prim<R> &Rt, R cr) {
  if constexpr (FA) return hf::hllc<AX>(k, L, cl, Rt, cr);
  else return hs::hllc<AX>(g, L, cl, Rt, cr);
}

// MUSCL face values in the exact or the production algebra
template <bool FA, class R>
__device__ __forceinline__ void muscl(R x0, R x1, R x2, R x3, R &l, R &r) {
  if constexpr (FA) hf::muscl(x0, x1, x2, x3, l, r);
  else hs::muscl(x0, x1, x2, x3, l, r);
}

// sound speed of a state in the exact or the production algebra
template <bool FA, class R>
__device__ __forceinline__ R face_sound(R g, const hf::Consts<R> &k, R rho, R p) {
  if constexpr (FA) return hf::sound(k, rho, p);
  else return hs::sound(g, rho, p);
}

template <bool FA, class R>
__device__ __forceinline__ hs::Prim<R> cell_update(R g, const hf::Consts<R> &k,
                                                   const hs::Prim<R> &b, R dtdx0, R dtdx1,
                                                   const hs::Flux<R> &l0, const hs::Flux<R> &r0,
                                                   const hs::Flux<R> &l1, const hs::Flux<R> &r1,
                                                   R *cons = nullptr) {
  if constexpr (FA) return hf::update(k, b, dtdx0, dtdx1, l0, r0, l1, r1, cons);
  else return hs::update(g, b, dtdx0, dtdx1, l0, r0, l1, r1, cons);
}

}  // namespace hk

// ---------------------------------------------------------------------------
// CFL timescale minimum of a state (used when no fused step has produced it)
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(256)
hydro_tsmin_kernel(const R *__restrict__ rho, const R *__restrict__ v0,
                   const R *__restrict__ v1, const R *__restrict__ p, size_t n,
                   double gamma, HydroScalars *sc, int slot) {
  __shared__ unsigned long long red[32];
  const R g = (R)gamma, dR0 = (R)sc->dR0, dR1 = (R)sc->dR1;
  unsigned long long m = ~0ull;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const R t = hs::timescale(g, dR0, dR1, rho[i], v0[i], v1[i], p[i]);
    const unsigned long long b = hk::ts_bits<R>(t);
    m = b < m ? b : m;
  }
  hk::block_min_to(m, &sc->tsmin[slot], red);
}

// ---------------------------------------------------------------------------
// Fused two-stage step on a TX x TY tile with a 3-cell cyclic halo.
// Phases: load (with sound speeds) -> stage-1 walls (order 1, one HLLC per
// face) -> stage-1 cells (dt/2) -> stage-2 walls (MUSCL + HLLC) -> stage-2
// cells (dt), written out with the tile's CFL minimum of the new state.
// ---------------------------------------------------------------------------
template <class R, int TX, int TY> struct FusedSmem {
  static constexpr int PX = TX + 6, PY = TY + 6;   // loaded cells
  static constexpr int QX = TX + 4, QY = TY + 4;   // stage-1 cells
  static constexpr int FXX = TX + 5, FXY = TY + 4; // stage-1 x walls
  static constexpr int FYX = TX + 4, FYY = TY + 5; // stage-1 y walls
  R P[4][PY][PX];
  R C[PY][PX];
  R Q[4][QY][QX];
  hs::Flux<R> fx[FXY * FXX];
  hs::Flux<R> fy[FYY * FYX];
};

// One tile of the fused step (tile index `tile` of the grid described by a),
// run by a whole block; the tile with index 0 advances the instance's time.
// OPEN: the grid has margins of width a.lm; box cells outside the interior
// take the jet state of the boundary condition instead of a periodic image,
// and the margin cells' timescale minimum joins the CFL minimum.
// TAPE (periodic grids): the tile's stage-1 states and both stages' flux
// differences are also written to `tape`.
// FA: the production algebra (hf::) instead of the generated order (hs::).
template <class R, int TX, int TY, int NT, bool OPEN = false, bool TAPE = false, bool FA = false>
__device__ __forceinline__ void fused_tile(const HydroStepArgs &a, int tile,
                                           FusedSmem<R, TX, TY> &s, unsigned long long *red,
                                           const HydroTapeOut *tape = nullptr) {
  using S = FusedSmem<R, TX, TY>;
  const int tid = threadIdx.x;
  const int t0 = tile % a.nt0, t1 = tile / a.nt0;
  const int X0 = t0 * TX, Y0 = t1 * TY;
  const int n0 = a.n0, n1 = a.n1;
  const R g = hk::Reals<R>::gamma(a);
  const hf::Consts<R> K = hf::consts<R>(g);
  const R dR0 = hk::Reals<R>::dR0(a.sc), dR1 = hk::Reals<R>::dR1(a.sc);
  const R dtG = hk::step_dt<R>(a);
  const R dtHalf = dtG / R(2);
  const R *rho = (const R *)a.rho, *vx = (const R *)a.v0, *vy = (const R *)a.v1,
          *pr = (const R *)a.p;

  // phase 0: load primitives and sound speeds.  Box indices run from -3 to
  // n + T + 1 (T the tile extent), inside [-n, 2n) once n >= T + 8.
  const bool near = n0 >= TX + 8 && n1 >= TY + 8;
  for (int i = tid; i < S::PY * S::PX; i += NT) {
    const int py = i / S::PX, px = i - py * S::PX;
    R r, u, v, q;
    if (OPEN) {
      const int ix = X0 + px - 3, iy = Y0 + py - 3;
      if (ix < 0 || iy < 0 || ix >= n0 || iy >= n1) {
        const hs::Prim<R> j = hk::jet_state<R>(g, dR0, dR1, hk::Reals<R>::ext1(a.sc), ix, iy);
        r = j.rho; u = j.v0; v = j.v1; q = j.p;
      } else {
        const size_t gi = (size_t)(iy + a.lm) * a.ms0 + (ix + a.lm);
        r = rho[gi]; u = vx[gi]; v = vy[gi]; q = pr[gi];
      }
    } else {
      const int gy = near ? hk::wrap_near(Y0 + py - 3, n1) : hk::wrap<R>(Y0 + py - 3, n1);
      const int gx = near ? hk::wrap_near(X0 + px - 3, n0) : hk::wrap<R>(X0 + px - 3, n0);
      const size_t gi = (size_t)gy * n0 + gx;
      r = rho[gi]; u = vx[gi]; v = vy[gi]; q = pr[gi];
    }
    s.P[0][py][px] = r;
    s.P[1][py][px] = u;
    s.P[2][py][px] = v;
    s.P[3][py][px] = q;
    s.C[py][px] = hk::face_sound<FA>(g, K, r, q);
  }
  __syncthreads();

  // phase 1: stage-1 walls, order-1 reconstruction (L = cell left, R = cell)
  {
    constexpr int NX = S::FXY * S::FXX, NY = S::FYY * S::FYX;
    for (int i = tid; i < NX + NY; i += NT) {
      if (i < NX) {
        const int fy = i / S::FXX, fx = i - fy * S::FXX;
        const int py = fy + 1;
        const hs::Prim<R> L{s.P[0][py][fx], s.P[1][py][fx], s.P[2][py][fx], s.P[3][py][fx]};
        const hs::Prim<R> Rt{s.P[0][py][fx + 1], s.P[1][py][fx + 1], s.P[2][py][fx + 1],
                             s.P[3][py][fx + 1]};
        s.fx[i] = hk::wall_flux<FA, 0>(g, K, L, s.C[py][fx], Rt, s.C[py][fx + 1]);
      } else {
        const int j = i - NX;
        const int fy = j / S::FYX, fx = j - fy * S::FYX;
        const int px = fx + 1;
        const hs::Prim<R> L{s.P[0][fy][px], s.P[1][fy][px], s.P[2][fy][px], s.P[3][fy][px]};
        const hs::Prim<R> Rt{s.P[0][fy + 1][px], s.P[1][fy + 1][px], s.P[2][fy + 1][px],
                             s.P[3][fy + 1][px]};
        s.fy[j] = hk::wall_flux<FA, 1>(g, K, L, s.C[fy][px], Rt, s.C[fy + 1][px]);
      }
    }
  }
  __syncthreads();

  // phase 2: stage-1 cells
  {
    const R dtdx0 = dtHalf / dR0, dtdx1 = dtHalf / dR1;
    for (int i = tid; i < S::QY * S::QX; i += NT) {
      const int qy = i / S::QX, qx = i - qy * S::QX;
      const int py = qy + 1, px = qx + 1;
      const hs::Prim<R> b{s.P[0][py][px], s.P[1][py][px], s.P[2][py][px], s.P[3][py][px]};
      const hs::Prim<R> q = hk::cell_update<FA>(g, K, b, dtdx0, dtdx1, s.fx[qy * S::FXX + qx],
                                                s.fx[qy * S::FXX + qx + 1], s.fy[qy * S::FYX + qx],
                                                s.fy[(qy + 1) * S::FYX + qx]);
      s.Q[0][qy][qx] = q.rho;
      s.Q[1][qy][qx] = q.v0;
      s.Q[2][qy][qx] = q.v1;
      s.Q[3][qy][qx] = q.p;
      if (TAPE) {
        const int ty = qy - 2, tx = qx - 2;
        if (ty >= 0 && ty < TY && tx >= 0 && tx < TX && Y0 + ty < n1 && X0 + tx < n0) {
          const size_t gi = (size_t)(Y0 + ty) * n0 + (X0 + tx);
          ((R *)tape->q[0])[gi] = q.rho;
          ((R *)tape->q[1])[gi] = q.v0;
          ((R *)tape->q[2])[gi] = q.v1;
          ((R *)tape->q[3])[gi] = q.p;
          hk::tape_diffs<R>(tape->d1, gi, s.fx[qy * S::FXX + qx], s.fx[qy * S::FXX + qx + 1],
                            s.fy[qy * S::FYX + qx], s.fy[(qy + 1) * S::FYX + qx]);
        }
      }
    }
  }
  __syncthreads();

  // phase 3: stage-2 walls with MUSCL-minmod reconstruction of stage-1 cells
  {
    constexpr int NX = TY * (TX + 1), NY = (TY + 1) * TX;
    for (int i = tid; i < NX + NY; i += NT) {
      hs::Prim<R> L, Rt;
      if (i < NX) {
        const int sy = i / (TX + 1), sx = i - sy * (TX + 1);
        const int qy = sy + 2;
#pragma unroll
        for (int f = 0; f < 4; ++f) {
          R l, r;
          hk::muscl<FA>(s.Q[f][qy][sx], s.Q[f][qy][sx + 1], s.Q[f][qy][sx + 2], s.Q[f][qy][sx + 3],
                    l, r);
          (&L.rho)[f] = l;
          (&Rt.rho)[f] = r;
        }
        s.fx[i] = hk::wall_flux<FA, 0>(g, K, L, hk::face_sound<FA>(g, K, L.rho, L.p), Rt,
                                       hk::face_sound<FA>(g, K, Rt.rho, Rt.p));
      } else {
        const int j = i - NX;
        const int sy = j / TX, sx = j - sy * TX;
        const int qx = sx + 2;
#pragma unroll
        for (int f = 0; f < 4; ++f) {
          R l, r;
          hk::muscl<FA>(s.Q[f][sy][qx], s.Q[f][sy + 1][qx], s.Q[f][sy + 2][qx], s.Q[f][sy + 3][qx],
                    l, r);
          (&L.rho)[f] = l;
          (&Rt.rho)[f] = r;
        }
        s.fy[j] = hk::wall_flux<FA, 1>(g, K, L, hk::face_sound<FA>(g, K, L.rho, L.p), Rt,
                                       hk::face_sound<FA>(g, K, Rt.rho, Rt.p));
      }
    }
  }
  __syncthreads();

  // phase 4: stage-2 cells, written out, with the CFL minimum of the new state
  unsigned long long m = ~0ull;
  {
    const R dtdx0 = dtG / dR0, dtdx1 = dtG / dR1;
    R *orho = (R *)a.nrho, *ovx = (R *)a.nv0, *ovy = (R *)a.nv1, *opr = (R *)a.np;
    for (int i = tid; i < TY * TX; i += NT) {
      const int oy = i / TX, ox = i - oy * TX;
      const int gy = Y0 + oy, gx = X0 + ox;
      if (gy >= n1 || gx >= n0) continue;
      const int py = oy + 3, px = ox + 3;
      const hs::Prim<R> b{s.P[0][py][px], s.P[1][py][px], s.P[2][py][px], s.P[3][py][px]};
      R cons[4];
      const hs::Prim<R> q = hk::cell_update<FA>(
          g, K, b, dtdx0, dtdx1, s.fx[oy * (TX + 1) + ox], s.fx[oy * (TX + 1) + ox + 1],
          s.fy[oy * TX + ox], s.fy[(oy + 1) * TX + ox], TAPE ? cons : nullptr);
      const size_t gi = OPEN ? (size_t)(gy + a.lm) * a.ms0 + (gx + a.lm) : (size_t)gy * n0 + gx;
      if (TAPE) {
        hk::tape_diffs<R>(tape->d2, gi, s.fx[oy * (TX + 1) + ox], s.fx[oy * (TX + 1) + ox + 1],
                          s.fy[oy * TX + ox], s.fy[(oy + 1) * TX + ox]);
#pragma unroll
        for (int c = 0; c < 4; ++c) ((R *)tape->u2[c])[gi] = cons[c];
      }
      orho[gi] = q.rho;
      ovx[gi] = q.v0;
      ovy[gi] = q.v1;
      opr[gi] = q.p;
      const R t = hs::timescale(g, dR0, dR1, q.rho, q.v0, q.v1, q.p);
      const unsigned long long bits = hk::ts_bits<R>(t);
      m = bits < m ? bits : m;
    }
  }
  if (OPEN) {
    // the generated class copies whole manifests, whose margins are zero,
    // into the statics: tiles on the grid edge clear the adjacent margins
    const int lm = a.lm;
    const int xa = X0 == 0 ? -lm : X0, xb = X0 + TX >= n0 ? n0 + lm : X0 + TX;
    const int ya = Y0 == 0 ? -lm : Y0, yb = Y0 + TY >= n1 ? n1 + lm : Y0 + TY;
    const int w = xb - xa, cnt = w * (yb - ya);
    if (xa < 0 || ya < 0 || xb > n0 || yb > n1) {
      R *orho = (R *)a.nrho, *ovx = (R *)a.nv0, *ovy = (R *)a.nv1, *opr = (R *)a.np;
      for (int i = tid; i < cnt; i += NT) {
        const int y = ya + i / w, x = xa + i % w;
        if (x >= 0 && y >= 0 && x < n0 && y < n1) continue;
        const size_t gi = (size_t)(y + lm) * a.ms0 + (x + lm);
        orho[gi] = R(0);
        ovx[gi] = R(0);
        ovy[gi] = R(0);
        opr[gi] = R(0);
      }
    }
  }
  hk::block_min_to(m, &a.sc->tsmin[1 - a.read_slot], red);
  if (OPEN && tile == 0 && tid == 0) atomicMin(&a.sc->tsmin[1 - a.read_slot], *a.margin_min);
  if (tile == 0 && tid == 0) {
    a.dt_hist[0] = (double)dtG;
    a.sc->dt_last = (double)dtG;
    a.sc->time = a.sc->time + (double)dtG;
  }
}

template <class R, int TX, int TY, int NT, bool OPEN = false, bool FA = false>
__global__ void __launch_bounds__(NT)
hydro_fused_kernel(HydroStepArgs a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long red[32];
  fused_tile<R, TX, TY, NT, OPEN, false, FA>(
      a, blockIdx.x, *reinterpret_cast<FusedSmem<R, TX, TY> *>(smem_raw), red);
}

// the fused step that also writes the tape of the reverse sweep (periodic)
template <class R, int TX, int TY, int NT, bool FA = false>
__global__ void __launch_bounds__(NT)
hydro_fused_tape_kernel(HydroStepArgs a, const __grid_constant__ HydroTapeOut t) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long red[32];
  fused_tile<R, TX, TY, NT, false, true, FA>(
      a, blockIdx.x, *reinterpret_cast<FusedSmem<R, TX, TY> *>(smem_raw), red, &t);
}

// CFL timescale minimum of the margin cells of an open grid (the jet state
// of the boundary condition; it depends only on the index, gamma, dR and
// extent1)
template <class R>
__global__ void __launch_bounds__(256)
hydro_margin_min_kernel(int n0, int n1, int lm, double gamma, const HydroScalars *sc,
                        unsigned long long *out) {
  __shared__ unsigned long long red[32];
  const R g = (R)gamma, dR0 = (R)sc->dR0, dR1 = (R)sc->dR1, ext1 = (R)sc->extent1;
  const int ms0 = n0 + 2 * lm, ms1 = n1 + 2 * lm;
  const size_t total = (size_t)ms0 * ms1;
  unsigned long long m = ~0ull;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / ms0), x = (int)(i - (size_t)y * ms0);
    const int ix = x - lm, iy = y - lm;
    if (ix >= 0 && iy >= 0 && ix < n0 && iy < n1) continue;
    const hs::Prim<R> q = hk::jet_state<R>(g, dR0, dR1, ext1, ix, iy);
    const unsigned long long b = hk::ts_bits<R>(hs::timescale(g, dR0, dR1, q.rho, q.v0, q.v1, q.p));
    m = b < m ? b : m;
  }
  hk::block_min_to(m, out, red);
}

// CFL minimum of an open grid's current state: the interior cells, then
// the margin cells' minimum
template <class R>
__global__ void __launch_bounds__(256)
hydro_tsmin_open_kernel(const R *__restrict__ rho, const R *__restrict__ v0,
                        const R *__restrict__ v1, const R *__restrict__ p, int n0, int n1, int lm,
                        double gamma, HydroScalars *sc, int slot,
                        const unsigned long long *margin_min) {
  __shared__ unsigned long long red[32];
  const R g = (R)gamma, dR0 = (R)sc->dR0, dR1 = (R)sc->dR1;
  const int ms0 = n0 + 2 * lm;
  const size_t n = (size_t)n0 * n1;
  unsigned long long m = ~0ull;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / n0), x = (int)(i - (size_t)y * n0);
    const size_t gi = (size_t)(y + lm) * ms0 + (x + lm);
    const R t = hs::timescale(g, dR0, dR1, rho[gi], v0[gi], v1[gi], p[gi]);
    const unsigned long long b = hk::ts_bits<R>(t);
    m = b < m ? b : m;
  }
  hk::block_min_to(m, &sc->tsmin[slot], red);
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicMin(&sc->tsmin[slot], *margin_min);
}

// Ensemble step: every tile of every instance is one work item; the
// persistent grid strides over the flattened item list (prefix[k] = first
// item of instance k), so instances of any size advance in one launch, each
// with its own dt, CFL minimum and time (its HydroStepArgs).  Up to
// kEnsPrefixShared instances, the prefix is kept in shared memory.
constexpr int kEnsPrefixShared = 1024;

template <class R, int TX, int TY, int NT, bool FA = false>
__global__ void __launch_bounds__(NT)
hydro_ensemble_kernel(const HydroStepArgs *__restrict__ args, const int *__restrict__ prefix,
                      int count) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long red[32];
  __shared__ int spref[kEnsPrefixShared + 1];
  auto &s = *reinterpret_cast<FusedSmem<R, TX, TY> *>(smem_raw);
  // a block's items increase, so its instance index only moves forward: it
  // advances through the prefix (in shared memory when it fits) instead of
  // searching global memory per item
  const bool shared = count <= kEnsPrefixShared;
  if (shared)
    for (int i = threadIdx.x; i <= count; i += NT) spref[i] = prefix[i];
  __syncthreads();
  const int *pf = shared ? spref : prefix;
  const int total = pf[count];
  int lo = 0;  // instance k with prefix[k] <= item < prefix[k+1]
  for (int item = blockIdx.x; item < total; item += gridDim.x) {
    while (lo < count - 1 && pf[lo + 1] <= item) ++lo;
    fused_tile<R, TX, TY, NT, false, false, FA>(args[lo], item - pf[lo], s, red);
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Plain path: the structure of the generated code.  One thread per cell,
// every Delayed value recomputed from the four primitive arrays in global
// memory (as Hydro_sub_8 does), grid-stride loops, separate timescale and
// reduce passes, and copies of the manifests back into the statics.
// ---------------------------------------------------------------------------
template <class R>
__global__ void __launch_bounds__(256)
hydro_plain_timescale_kernel(const R *__restrict__ rho, const R *__restrict__ v0,
                             const R *__restrict__ v1, const R *__restrict__ p,
                             R *__restrict__ ts, size_t n, double gamma,
                             const HydroScalars *sc) {
  const R g = (R)gamma, dR0 = (R)sc->dR0, dR1 = (R)sc->dR1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x)
    ts[i] = hs::timescale(g, dR0, dR1, rho[i], v0[i], v1[i], p[i]);
}

template <class R>
__global__ void __launch_bounds__(256)
hydro_plain_reduce_min_kernel(const R *__restrict__ ts, size_t n, unsigned long long *out) {
  __shared__ unsigned long long red[32];
  unsigned long long m = ~0ull;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const unsigned long long b = hk::ts_bits<R>(ts[i]);
    m = b < m ? b : m;
  }
  hk::block_min_to(m, out, red);
}

template <class R> struct PlainView {
  const R *rho, *v0, *v1, *p;
  int n0, n1;
  __device__ __forceinline__ hs::Prim<R> at(int x, int y) const {
    x = hk::wrap<R>(x, n0);
    y = hk::wrap<R>(y, n1);
    const size_t i = (size_t)y * n0 + x;
    return hs::Prim<R>{rho[i], v0[i], v1[i], p[i]};
  }
};

// stage-1 state at (x, y): order-1 walls recomputed from the primitives
template <class R>
__device__ __forceinline__ hs::Prim<R> plain_stage1(const PlainView<R> &V, R g, R dtdx0, R dtdx1,
                                                    int x, int y) {
  const hs::Prim<R> c = V.at(x, y), xm = V.at(x - 1, y), xp = V.at(x + 1, y),
                    ym = V.at(x, y - 1), yp = V.at(x, y + 1);
  const R cc = hs::sound(g, c.rho, c.p);
  const hs::Flux<R> l0 = hs::hllc<0>(g, xm, hs::sound(g, xm.rho, xm.p), c, cc);
  const hs::Flux<R> r0 = hs::hllc<0>(g, c, cc, xp, hs::sound(g, xp.rho, xp.p));
  const hs::Flux<R> l1 = hs::hllc<1>(g, ym, hs::sound(g, ym.rho, ym.p), c, cc);
  const hs::Flux<R> r1 = hs::hllc<1>(g, c, cc, yp, hs::sound(g, yp.rho, yp.p));
  return hs::update(g, c, dtdx0, dtdx1, l0, r0, l1, r1);
}

template <int AX, class R>
__device__ __forceinline__ hs::Flux<R> plain_wall2(const hs::Prim<R> &a0, const hs::Prim<R> &a1,
                                                   const hs::Prim<R> &a2, const hs::Prim<R> &a3,
                                                   R g) {
  hs::Prim<R> L, Rt;
  hs::muscl(a0.rho, a1.rho, a2.rho, a3.rho, L.rho, Rt.rho);
  hs::muscl(a0.v0, a1.v0, a2.v0, a3.v0, L.v0, Rt.v0);
  hs::muscl(a0.v1, a1.v1, a2.v1, a3.v1, L.v1, Rt.v1);
  hs::muscl(a0.p, a1.p, a2.p, a3.p, L.p, Rt.p);
  return hs::hllc<AX>(g, L, hs::sound(g, L.rho, L.p), Rt, hs::sound(g, Rt.rho, Rt.p));
}

template <class R>
__global__ void __launch_bounds__(128)
hydro_plain_step_kernel(PlainView<R> V, R *__restrict__ orho, R *__restrict__ ov0,
                        R *__restrict__ ov1, R *__restrict__ op, double gamma, R dtG, R dR0,
                        R dR1) {
  const R g = (R)gamma;
  const R dtHalf = dtG / R(2);
  const R h0 = dtHalf / dR0, h1 = dtHalf / dR1;
  const R f0 = dtG / dR0, f1 = dtG / dR1;
  const size_t n = (size_t)V.n0 * V.n1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / V.n0), x = (int)(i - (size_t)y * V.n0);
    // stage-1 cells along the two axes (Delayed: recomputed here)
    const hs::Prim<R> qm2 = plain_stage1(V, g, h0, h1, x - 2, y);
    const hs::Prim<R> qm1 = plain_stage1(V, g, h0, h1, x - 1, y);
    const hs::Prim<R> q00 = plain_stage1(V, g, h0, h1, x, y);
    const hs::Prim<R> qp1 = plain_stage1(V, g, h0, h1, x + 1, y);
    const hs::Prim<R> qp2 = plain_stage1(V, g, h0, h1, x + 2, y);
    const hs::Flux<R> l0 = plain_wall2<0>(qm2, qm1, q00, qp1, g);
    const hs::Flux<R> r0 = plain_wall2<0>(qm1, q00, qp1, qp2, g);
    const hs::Prim<R> ym2 = plain_stage1(V, g, h0, h1, x, y - 2);
    const hs::Prim<R> ym1 = plain_stage1(V, g, h0, h1, x, y - 1);
    const hs::Prim<R> yp1 = plain_stage1(V, g, h0, h1, x, y + 1);
    const hs::Prim<R> yp2 = plain_stage1(V, g, h0, h1, x, y + 2);
    const hs::Flux<R> l1 = plain_wall2<1>(ym2, ym1, q00, yp1, g);
    const hs::Flux<R> r1 = plain_wall2<1>(ym1, q00, yp1, yp2, g);
    const hs::Prim<R> q = hs::update(g, V.at(x, y), f0, f1, l0, r0, l1, r1);
    orho[i] = q.rho;
    ov0[i] = q.v0;
    ov1[i] = q.v1;
    op[i] = q.p;
  }
}

}  // namespace om

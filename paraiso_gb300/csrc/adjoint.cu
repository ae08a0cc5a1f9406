// adjoint.cu -- reverse-mode adjoint of the Hydro step on GB300 (no
// counterpart in the reference; the forward is examples/Hydro/HydroMain.hs
// proceed, HydroMain.hs:134-164).
//
// One adjoint step maps the cotangent of the state after a step to the
// cotangent of the state before it, through both stages, both axes, the
// MUSCL-minmod reconstruction, the HLLC fluxes, the clamps and the dt of the
// step (dt = cfl * min timescale: its cotangent is routed to the arg-min
// cell).  The step is a sequence of gather kernels over cells and faces, so
// every cotangent is written by exactly one thread:
//   A  stage-1 state Q (forward recompute)
//   B  per cell: stage-2 update reverse -> conserved cotangent U2b, base part
//   C  per face: stage-2 flux cotangent -> HLLC and reconstruction inputs
//   D  per cell: gather into Qb; stage-1 update reverse -> U1b, base part
//   E  per face: stage-1 flux cotangent -> HLLC inputs
//   F  per cell: gather the stage-1 face cotangents into the base cotangent
//   G  the dt cotangent (block partials summed in order) to the arg-min cell
// Multi-step gradients use sqrt(T) checkpointing: the forward keeps every
// s-th state, the backward recomputes each segment and walks it backwards.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "hydro_adjoint.cuh"
#include "hydro_launch.cuh"
#include "om_internal.cuh"

namespace om {
namespace adj {

using ha::PrimBar;
using hs::Flux;
using hs::Prim;

template <class R> struct Fields {
  R *f[4];
  __device__ __forceinline__ Prim<R> get(size_t i) const {
    return Prim<R>{f[0][i], f[1][i], f[2][i], f[3][i]};
  }
  __device__ __forceinline__ void set(size_t i, const Prim<R> &q) const {
    f[0][i] = q.rho; f[1][i] = q.v0; f[2][i] = q.v1; f[3][i] = q.p;
  }
};

template <class R> struct Geo {
  int n0, n1;
  R g, dR0, dR1, dt;
  const double *dtp;  // the step's dt in device memory (read at kernel start)
  // periodic index of a cell at most 4 cells outside the mesh
  __device__ __forceinline__ size_t at(int x, int y) const {
    if (n0 >= 8 && n1 >= 8) {
      x += x < 0 ? n0 : 0;
      x -= x >= n0 ? n0 : 0;
      y += y < 0 ? n1 : 0;
      y -= y >= n1 ? n1 : 0;
    } else {
      x %= n0; if (x < 0) x += n0;
      y %= n1; if (y < 0) y += n1;
    }
    return (size_t)y * n0 + x;
  }
};

// one stored flux per face and axis: 4 arrays per axis
template <class R> struct FluxStore {
  R *f[8];  // axis 0: fd, fm0, fm1, fe; axis 1: fd, fm0, fm1, fe
  __device__ __forceinline__ Flux<R> get(int ax, size_t i) const {
    return Flux<R>{f[4 * ax][i], f[4 * ax + 1][i], f[4 * ax + 2][i], f[4 * ax + 3][i]};
  }
  __device__ __forceinline__ void set(int ax, size_t i, const Flux<R> &v) const {
    f[4 * ax][i] = v.fd; f[4 * ax + 1][i] = v.fm0; f[4 * ax + 2][i] = v.fm1; f[4 * ax + 3][i] = v.fe;
  }
};

// order-1 stage-1 wall along AX at cell (x, y): between (x,y)-e and (x,y)
template <int AX, class R>
__device__ __forceinline__ Flux<R> wall1(const Fields<R> &P, const Geo<R> &G, int x, int y) {
  const Prim<R> L = AX == 0 ? P.get(G.at(x - 1, y)) : P.get(G.at(x, y - 1));
  const Prim<R> Rt = P.get(G.at(x, y));
  return hs::hllc<AX>(G.g, L, hs::sound(G.g, L.rho, L.p), Rt, hs::sound(G.g, Rt.rho, Rt.p));
}

// MUSCL face states of the stage-2 wall along AX at (x, y)
template <int AX, class R>
__device__ __forceinline__ void face2_states(const Fields<R> &Q, const Geo<R> &G, int x, int y,
                                             Prim<R> &L, Prim<R> &Rt, Prim<R> st[4]) {
#pragma unroll
  for (int k = 0; k < 4; ++k)
    st[k] = AX == 0 ? Q.get(G.at(x - 2 + k, y)) : Q.get(G.at(x, y - 2 + k));
  hs::muscl(st[0].rho, st[1].rho, st[2].rho, st[3].rho, L.rho, Rt.rho);
  hs::muscl(st[0].v0, st[1].v0, st[2].v0, st[3].v0, L.v0, Rt.v0);
  hs::muscl(st[0].v1, st[1].v1, st[2].v1, st[3].v1, L.v1, Rt.v1);
  hs::muscl(st[0].p, st[1].p, st[2].p, st[3].p, L.p, Rt.p);
}

template <int AX, class R>
__device__ __forceinline__ Flux<R> wall2(const Fields<R> &Q, const Geo<R> &G, int x, int y) {
  Prim<R> L, Rt, st[4];
  face2_states<AX>(Q, G, x, y, L, Rt, st);
  return hs::hllc<AX>(G.g, L, hs::sound(G.g, L.rho, L.p), Rt, hs::sound(G.g, Rt.rho, Rt.p));
}

__device__ __forceinline__ double block_sum(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double t = 0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sh[w];
  __syncthreads();
  return t;
}

// A1: stage-1 walls, one per face and axis (face i: left wall of cell i)
template <class R>
__global__ void __launch_bounds__(256)
adj_walls1(Fields<R> P, FluxStore<R> F1, Geo<R> G, unsigned long long *minbits) {
  const size_t n = (size_t)G.n0 * G.n1;
  unsigned long long best = ~0ull;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / G.n0), x = (int)(i - (size_t)y * G.n0);
    F1.set(0, i, wall1<0>(P, G, x, y));
    F1.set(1, i, wall1<1>(P, G, x, y));
    const Prim<R> q = P.get(i);
    const unsigned long long b = hk::ts_bits<R>(hs::timescale(G.g, G.dR0, G.dR1, q.rho, q.v0,
                                                              q.v1, q.p));
    best = b < best ? b : best;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, best, o);
    best = w < best ? w : best;
  }
  if ((threadIdx.x & 31) == 0) atomicMin(minbits, best);
}

// A2: stage-1 state from the stored walls
template <class R>
__global__ void __launch_bounds__(256)
adj_stage1(Fields<R> P, FluxStore<R> F1, Fields<R> Q, Geo<R> G,
           const unsigned long long *minbits, unsigned long long *argmin) {
  G.dt = (R)*G.dtp;
  const size_t n = (size_t)G.n0 * G.n1;
  const R h = G.dt / R(2);
  const R d0 = h / G.dR0, d1 = h / G.dR1;
  const unsigned long long mb = *minbits;
  unsigned long long best = ~0ull;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / G.n0), x = (int)(i - (size_t)y * G.n0);
    const Prim<R> b = P.get(i);
    Q.set(i, hs::update(G.g, b, d0, d1, F1.get(0, i), F1.get(0, G.at(x + 1, y)),
                        F1.get(1, i), F1.get(1, G.at(x, y + 1))));
    const R t = hs::timescale(G.g, G.dR0, G.dR1, b.rho, b.v0, b.v1, b.p);
    if (hk::ts_bits<R>(t) == mb && i < best) best = i;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, best, o);
    best = w < best ? w : best;
  }
  if ((threadIdx.x & 31) == 0 && best != ~0ull) atomicMin(argmin, best);
}

// A3: stage-2 walls (MUSCL on the stage-1 state), one per face and axis
template <class R>
__global__ void __launch_bounds__(256) adj_walls2(Fields<R> Q, FluxStore<R> F2, Geo<R> G) {
  const size_t n = (size_t)G.n0 * G.n1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / G.n0), x = (int)(i - (size_t)y * G.n0);
    F2.set(0, i, wall2<0>(Q, G, x, y));
    F2.set(1, i, wall2<1>(Q, G, x, y));
  }
}

// B: stage-2 update reverse per cell
template <class R>
__global__ void __launch_bounds__(256)
adj_stage2_cells(Fields<R> P, FluxStore<R> F2, Fields<R> Ub, Fields<R> U2b, Fields<R> Pbase,
                 Geo<R> G, double *partial) {
  G.dt = (R)*G.dtp;
  __shared__ double sh[8];
  const size_t n = (size_t)G.n0 * G.n1;
  const R d0 = G.dt / G.dR0, d1 = G.dt / G.dR1;
  const R rdR0 = R(1) / G.dR0, rdR1 = R(1) / G.dR1;
  double dtb = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / G.n0), x = (int)(i - (size_t)y * G.n0);
    const Flux<R> l0 = F2.get(0, i), r0 = F2.get(0, G.at(x + 1, y));
    const Flux<R> l1 = F2.get(1, i), r1 = F2.get(1, G.at(x, y + 1));
    const Prim<R> b = P.get(i);
    R u[4];
    ha::update_cons(G.g, b, d0, d1, l0, r0, l1, r1, u);
    const Prim<R> qb_ = Ub.get(i);
    const PrimBar<R> qb{qb_.rho, qb_.v0, qb_.v1, qb_.p};
    R U[4];
    ha::cons_from_prim_rev(G.g, u[0], u[1], u[2], u[3], qb, U);
    U2b.set(i, Prim<R>{U[0], U[1], U[2], U[3]});
    PrimBar<R> bb;
    ha::zero(bb);
    ha::cons_of_prim_rev(G.g, b, U, bb);
    Pbase.set(i, Prim<R>{bb.rho, bb.v0, bb.v1, bb.p});
    const R t0 = U[0] * (l0.fd - r0.fd) + U[1] * (l0.fm0 - r0.fm0) + U[2] * (l0.fm1 - r0.fm1) +
                 U[3] * (l0.fe - r0.fe);
    const R t1 = U[0] * (l1.fd - r1.fd) + U[1] * (l1.fm0 - r1.fm0) + U[2] * (l1.fm1 - r1.fm1) +
                 U[3] * (l1.fe - r1.fe);
    dtb += (double)(t0 * rdR0 + t1 * rdR1);
  }
  const double s = block_sum(dtb, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// face cotangents of one axis: 8 arrays (L rho,v0,v1,p, R rho,v0,v1,p)
template <class R> struct FaceBar {
  R *f[8];
};

// reconstruction cotangents of one axis: slot k (0..3) of the stencil of
// face f (cells f-2 .. f+1), per field: 16 arrays
template <class R> struct SlotBar {
  R *f[16];  // [k * 4 + field]
};

// C: stage-2 walls reverse; face i along AX is the left wall of cell i and
// the right wall of cell i - e.  The HLLC reverse gives the cotangents of the
// reconstructed face states; the MUSCL reverse spreads them over the four
// stencil cells, stored per stencil slot for the gather in D.
template <class R>
__global__ void __launch_bounds__(256, 3)
adj_stage2_faces(Fields<R> Q, Fields<R> U2b, SlotBar<R> SX, SlotBar<R> SY, Geo<R> G) {
  G.dt = (R)*G.dtp;
  const size_t n = (size_t)G.n0 * G.n1;
  const R d0 = G.dt / G.dR0, d1 = G.dt / G.dR1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / G.n0), x = (int)(i - (size_t)y * G.n0);
#pragma unroll
    for (int ax = 0; ax < 2; ++ax) {
      const size_t im = ax == 0 ? G.at(x - 1, y) : G.at(x, y - 1);
      const R dd = ax == 0 ? d0 : d1;
      const Prim<R> a = U2b.get(i), c = U2b.get(im);
      const Flux<R> fb{dd * (a.rho - c.rho), dd * (a.v0 - c.v0), dd * (a.v1 - c.v1),
                       dd * (a.p - c.p)};
      Prim<R> L, Rt, st[4];
      PrimBar<R> Lb, Rb;
      ha::zero(Lb);
      ha::zero(Rb);
      if (ax == 0) {
        face2_states<0>(Q, G, x, y, L, Rt, st);
        ha::hllc_rev<0>(G.g, L, Rt, fb, Lb, Rb);
      } else {
        face2_states<1>(Q, G, x, y, L, Rt, st);
        ha::hllc_rev<1>(G.g, L, Rt, fb, Lb, Rb);
      }
      SlotBar<R> &S = ax == 0 ? SX : SY;
      const R lb[4] = {Lb.rho, Lb.v0, Lb.v1, Lb.p}, rb[4] = {Rb.rho, Rb.v0, Rb.v1, Rb.p};
#pragma unroll
      for (int c4 = 0; c4 < 4; ++c4) {
        R xb[4] = {0, 0, 0, 0};
        const R *xs = &st[0].rho;
        ha::muscl_rev((&st[0].rho)[c4], (&st[1].rho)[c4], (&st[2].rho)[c4], (&st[3].rho)[c4],
                      lb[c4], rb[c4], xb[0], xb[1], xb[2], xb[3]);
        (void)xs;
#pragma unroll
        for (int k = 0; k < 4; ++k) S.f[k * 4 + c4][i] = xb[k];
      }
    }
  }
}

// D: gather the reconstruction cotangents into Qb (face f = q + df holds this
// cell in stencil slot 2 - df), then stage-1 update reverse
template <class R>
__global__ void __launch_bounds__(256)
adj_stage1_cells(Fields<R> P, FluxStore<R> F1, SlotBar<R> SX, SlotBar<R> SY, Fields<R> U1b,
                 Fields<R> Pbase, Geo<R> G, double *partial) {
  G.dt = (R)*G.dtp;
  __shared__ double sh[8];
  const size_t n = (size_t)G.n0 * G.n1;
  const R h = G.dt / R(2);
  const R d0 = h / G.dR0, d1 = h / G.dR1;
  const R rdR0 = R(1) / G.dR0, rdR1 = R(1) / G.dR1;
  double dtb = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / G.n0), x = (int)(i - (size_t)y * G.n0);
    R qb[4] = {0, 0, 0, 0};
#pragma unroll
    for (int df = -1; df <= 2; ++df) {
      const size_t fx = G.at(x + df, y), fy = G.at(x, y + df);
      const int k = 2 - df;
#pragma unroll
      for (int c = 0; c < 4; ++c) qb[c] += SX.f[k * 4 + c][fx] + SY.f[k * 4 + c][fy];
    }
    const Flux<R> l0 = F1.get(0, i), r0 = F1.get(0, G.at(x + 1, y));
    const Flux<R> l1 = F1.get(1, i), r1 = F1.get(1, G.at(x, y + 1));
    const Prim<R> b = P.get(i);
    R u[4];
    ha::update_cons(G.g, b, d0, d1, l0, r0, l1, r1, u);
    const PrimBar<R> qbar{qb[0], qb[1], qb[2], qb[3]};
    R U[4];
    ha::cons_from_prim_rev(G.g, u[0], u[1], u[2], u[3], qbar, U);
    U1b.set(i, Prim<R>{U[0], U[1], U[2], U[3]});
    PrimBar<R> bb;
    const Prim<R> pb0 = Pbase.get(i);
    bb.rho = pb0.rho; bb.v0 = pb0.v0; bb.v1 = pb0.v1; bb.p = pb0.p;
    ha::cons_of_prim_rev(G.g, b, U, bb);
    Pbase.set(i, Prim<R>{bb.rho, bb.v0, bb.v1, bb.p});
    const R t0 = U[0] * (l0.fd - r0.fd) + U[1] * (l0.fm0 - r0.fm0) + U[2] * (l0.fm1 - r0.fm1) +
                 U[3] * (l0.fe - r0.fe);
    const R t1 = U[0] * (l1.fd - r1.fd) + U[1] * (l1.fm0 - r1.fm0) + U[2] * (l1.fm1 - r1.fm1) +
                 U[3] * (l1.fe - r1.fe);
    // dtdx = (dt / 2) / dR
    dtb += (double)(R(0.5) * (t0 * rdR0 + t1 * rdR1));
  }
  const double s = block_sum(dtb, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// E: stage-1 walls reverse
template <class R>
__global__ void __launch_bounds__(256, 3)
adj_stage1_faces(Fields<R> P, Fields<R> U1b, FaceBar<R> FX, FaceBar<R> FY, Geo<R> G) {
  G.dt = (R)*G.dtp;
  const size_t n = (size_t)G.n0 * G.n1;
  const R h = G.dt / R(2);
  const R d0 = h / G.dR0, d1 = h / G.dR1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / G.n0), x = (int)(i - (size_t)y * G.n0);
#pragma unroll
    for (int ax = 0; ax < 2; ++ax) {
      const size_t im = ax == 0 ? G.at(x - 1, y) : G.at(x, y - 1);
      const R dd = ax == 0 ? d0 : d1;
      const Prim<R> a = U1b.get(i), c = U1b.get(im);
      const Flux<R> fb{dd * (a.rho - c.rho), dd * (a.v0 - c.v0), dd * (a.v1 - c.v1),
                       dd * (a.p - c.p)};
      const Prim<R> L = P.get(im), Rt = P.get(i);
      PrimBar<R> Lb, Rb;
      ha::zero(Lb);
      ha::zero(Rb);
      if (ax == 0) ha::hllc_rev<0>(G.g, L, Rt, fb, Lb, Rb);
      else ha::hllc_rev<1>(G.g, L, Rt, fb, Lb, Rb);
      FaceBar<R> &F = ax == 0 ? FX : FY;
      F.f[0][i] = Lb.rho; F.f[1][i] = Lb.v0; F.f[2][i] = Lb.v1; F.f[3][i] = Lb.p;
      F.f[4][i] = Rb.rho; F.f[5][i] = Rb.v0; F.f[6][i] = Rb.v1; F.f[7][i] = Rb.p;
    }
  }
}

// F: previous-state cotangent = base part + stage-1 walls (the cell is the
// right state of its own wall and the left state of the next wall)
template <class R>
__global__ void __launch_bounds__(256)
adj_gather(Fields<R> Pbase, FaceBar<R> FX, FaceBar<R> FY, Fields<R> Pb, Geo<R> G) {
  const size_t n = (size_t)G.n0 * G.n1;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / G.n0), x = (int)(i - (size_t)y * G.n0);
    const size_t ix = G.at(x + 1, y), iy = G.at(x, y + 1);
    Prim<R> b = Pbase.get(i);
    b.rho += FX.f[4][i] + FX.f[0][ix] + FY.f[4][i] + FY.f[0][iy];
    b.v0 += FX.f[5][i] + FX.f[1][ix] + FY.f[5][i] + FY.f[1][iy];
    b.v1 += FX.f[6][i] + FX.f[2][ix] + FY.f[6][i] + FY.f[2][iy];
    b.p += FX.f[7][i] + FX.f[3][ix] + FY.f[7][i] + FY.f[3][iy];
    Pb.set(i, b);
  }
}

// G: dt cotangent to the arg-min cell.  The block partials are summed by one
// block in a fixed order (strided per thread, then a fixed tree), so the
// result does not depend on scheduling.
template <class R>
__global__ void __launch_bounds__(256)
adj_dt(Fields<R> P, Fields<R> Pb, Geo<R> G, const double *partials, int nparts, R cfl,
       const unsigned long long *argmin, double *dtb_out) {
  __shared__ double sh[256];
  double acc = 0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) acc += partials[k];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  const double dtb = sh[0];
  if (dtb_out) *dtb_out = dtb;
  const unsigned long long j = *argmin;
  if (j == ~0ull) return;
  const R tb = (R)(dtb * (double)cfl);
  PrimBar<R> xb;
  ha::zero(xb);
  ha::timescale_rev(G.g, G.dR0, G.dR1, P.get(j), tb, xb);
  Prim<R> b = Pb.get(j);
  b.rho += xb.rho; b.v0 += xb.v0; b.v1 += xb.v1; b.p += xb.p;
  Pb.set(j, b);
}

// loss = mean((rho - target)^2) and its cotangent 2 (rho - target) / N
template <class R>
__global__ void __launch_bounds__(256)
adj_loss(const R *rho, const R *target, R *rhob, size_t n, double *partial) {
  __shared__ double sh[8];
  double acc = 0;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const double d = (double)rho[i] - (double)target[i];
    acc += d * d;
    rhob[i] = (R)(2.0 * d / (double)n);
  }
  const double s = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

}  // namespace adj

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct AdjointScratch {
  int fp64 = -1;
  size_t cells = 0;
  void *q[4], *u2b[4], *u1b[4], *pbase[4], *fx[8], *fy[8], *ub[4], *pb[4], *f1[8], *f2[8];
  void *sx[16], *sy[16];
  void *stage[4];                 // the state a graph-captured step reads
  double *d_dt = nullptr;         // dt of the step being reversed
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // by cotangent buffer parity
  void *graph_ub[2] = {nullptr, nullptr};
  double graph_scalars[2][3] = {};  // cfl, dR0, dR1 each graph was captured with
  double *partials = nullptr;
  unsigned long long *argmin = nullptr;
  int nparts = 0;
  std::vector<void *> all;
};

static void free_scratch(AdjointScratch *s) {
  if (!s) return;
  for (int k = 0; k < 2; ++k)
    if (s->graph[k]) cudaGraphExecDestroy(s->graph[k]);
  cudaFree(s->d_dt);
  for (void *p : s->all) cudaFree(p);
  cudaFree(s->partials);
  cudaFree(s->argmin);
  delete s;
}

// scratch hangs off the handle's kind state through a small registry
static std::vector<std::pair<Handle *, AdjointScratch *>> g_scratch;

static om_status get_scratch(Handle *h, int fp64, AdjointScratch **out) {
  for (auto &kv : g_scratch)
    if (kv.first == h) {
      *out = kv.second;
      return OM_OK;
    }
  AdjointScratch *s = new AdjointScratch();
  s->fp64 = fp64;
  s->cells = h->memory_size_total();
  const size_t bytes = s->cells * (fp64 ? 8 : 4);
  void **groups[13] = {s->q,  s->u2b, s->u1b, s->pbase, s->ub, s->pb,   s->fx,
                       s->fy, s->f1,  s->f2,  s->sx,    s->sy, s->stage};
  const int sizes[13] = {4, 4, 4, 4, 4, 4, 8, 8, 8, 8, 16, 16, 4};
  for (int gi = 0; gi < 13; ++gi)
    for (int k = 0; k < sizes[gi]; ++k) {
      void *p = nullptr;
      if (cudaMalloc(&p, bytes) != cudaSuccess) {
        cudaGetLastError();
        free_scratch(s);
        set_error("Hydro adjoint: scratch allocation failed");
        return OM_ERR_NOMEM;
      }
      groups[gi][k] = p;
      s->all.push_back(p);
    }
  s->nparts = 2 * sm_count(h->device) * 4;
  if (cudaMalloc(&s->partials, sizeof(double) * 2 * s->nparts) != cudaSuccess ||
      cudaMalloc(&s->d_dt, sizeof(double)) != cudaSuccess ||
      cudaMalloc(&s->argmin, 2 * sizeof(unsigned long long)) != cudaSuccess) {
    cudaGetLastError();
    free_scratch(s);
    set_error("Hydro adjoint: scratch allocation failed");
    return OM_ERR_NOMEM;
  }
  g_scratch.push_back({h, s});
  *out = s;
  return OM_OK;
}

void adjoint_release(Handle *h) {
  for (size_t i = 0; i < g_scratch.size(); ++i)
    if (g_scratch[i].first == h) {
      free_scratch(g_scratch[i].second);
      g_scratch.erase(g_scratch.begin() + i);
      return;
    }
}

template <class R> static adj::Fields<R> F4(void *const *p) {
  return adj::Fields<R>{{(R *)p[0], (R *)p[1], (R *)p[2], (R *)p[3]}};
}

template <class R> static adj::FaceBar<R> F8(void *const *p) {
  adj::FaceBar<R> f;
  for (int k = 0; k < 8; ++k) f.f[k] = (R *)p[k];
  return f;
}

template <class R> static adj::SlotBar<R> S16(void *const *p) {
  adj::SlotBar<R> f;
  for (int k = 0; k < 16; ++k) f.f[k] = (R *)p[k];
  return f;
}

template <class R> static adj::FluxStore<R> FS(void *const *p) {
  adj::FluxStore<R> f;
  for (int k = 0; k < 8; ++k) f.f[k] = (R *)p[k];
  return f;
}

// One adjoint step at state `state` (4 device arrays) with step dt (in R)
// and CFL minimum bits: ub (4 device arrays, cotangent of the next state)
// -> pb_out (4 device arrays).  Returns the dt cotangent when dtb_out.
template <class R>
static om_status vjp_kernels(Handle *h, AdjointScratch *s, void *const *state, void *const *ub,
                             void *const *pb_out, double cfl, unsigned long long tsbits,
                             double *dtb_dev) {
  const cudaStream_t st = h->stream;
  const HydroScalars *hs_ = (const HydroScalars *)h->h_scalars;
  adj::Geo<R> G{h->size[0], h->size[1], (R)h->cfg.gamma, (R)hs_->dR0, (R)hs_->dR1, R(0), s->d_dt};
  const int grid = s->nparts;
  const auto P = F4<R>(state), Q = F4<R>(s->q), U = F4<R>(ub), U2b = F4<R>(s->u2b),
             U1b = F4<R>(s->u1b), Pbase = F4<R>(s->pbase), Pb = F4<R>(pb_out);
  const auto FX = F8<R>(s->fx), FY = F8<R>(s->fy);
  const auto F1 = FS<R>(s->f1), F2 = FS<R>(s->f2);
  const auto SX = S16<R>(s->sx), SY = S16<R>(s->sy);
  (void)tsbits;
  OM_CUDA_CHECK(cudaMemsetAsync(s->argmin, 0xFF, 2 * sizeof(unsigned long long), st));
  adj::adj_walls1<R><<<grid, 256, 0, st>>>(P, F1, G, s->argmin + 1);
  adj::adj_stage1<R><<<grid, 256, 0, st>>>(P, F1, Q, G, s->argmin + 1, s->argmin);
  adj::adj_walls2<R><<<grid, 256, 0, st>>>(Q, F2, G);
  adj::adj_stage2_cells<R><<<grid, 256, 0, st>>>(P, F2, U, U2b, Pbase, G, s->partials);
  adj::adj_stage2_faces<R><<<grid, 256, 0, st>>>(Q, U2b, SX, SY, G);
  adj::adj_stage1_cells<R><<<grid, 256, 0, st>>>(P, F1, SX, SY, U1b, Pbase, G,
                                                 s->partials + grid);
  adj::adj_stage1_faces<R><<<grid, 256, 0, st>>>(P, U1b, FX, FY, G);
  adj::adj_gather<R><<<grid, 256, 0, st>>>(Pbase, FX, FY, Pb, G);
  adj::adj_dt<R><<<1, 256, 0, st>>>(P, Pb, G, s->partials, 2 * grid, (R)cfl, s->argmin, dtb_dev);
  OM_CUDA_CHECK(cudaGetLastError());
  return OM_OK;
}

// One adjoint step on caller buffers without a graph (synchronous dt upload)
template <class R>
static om_status vjp_kernels_direct(Handle *h, AdjointScratch *s, void *const *state,
                                    void *const *ub, void *const *pb_out, double dt, double cfl,
                                    unsigned long long tsbits) {
  OM_CUDA_CHECK(cudaMemcpyAsync(s->d_dt, &dt, sizeof(double), cudaMemcpyHostToDevice, h->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  OM_TRY(vjp_kernels<R>(h, s, state, ub, pb_out, cfl, tsbits, nullptr));
  h->launches += 9;
  return OM_OK;
}

// One adjoint step: the step's dt (from host memory that stays untouched
// until the stream has read it) and the state go to fixed device buffers,
// then the kernel sequence runs from a CUDA graph captured once per
// cotangent buffer pair.
template <class R>
static om_status vjp_step(Handle *h, AdjointScratch *s, void *const *state, void *const *ub,
                          void *const *pb_out, const double *dt_host, double cfl,
                          unsigned long long tsbits, double *dtb_dev) {
  const cudaStream_t st = h->stream;
  const size_t bytes = s->cells * sizeof(R);
  OM_CUDA_CHECK(cudaMemcpyAsync(s->d_dt, dt_host, sizeof(double), cudaMemcpyHostToDevice, st));
  for (int k = 0; k < 4; ++k)
    if (state[k] != s->stage[k])
      OM_CUDA_CHECK(cudaMemcpyAsync(s->stage[k], state[k], bytes, cudaMemcpyDeviceToDevice, st));
  const int key = ub[0] == s->ub[0] ? 0 : 1;
  // scalars baked into the captured kernel arguments
  const HydroScalars *hs_ = (const HydroScalars *)h->h_scalars;
  const double baked[3] = {cfl, hs_->dR0, hs_->dR1};
  if (!s->graph[key] || s->graph_ub[key] != ub[0] ||
      std::memcmp(baked, s->graph_scalars[key], sizeof(baked)) != 0) {
    if (s->graph[key]) cudaGraphExecDestroy(s->graph[key]);
    s->graph[key] = nullptr;
    cudaGraph_t g = nullptr;
    OM_CUDA_CHECK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    om_status r = vjp_kernels<R>(h, s, s->stage, ub, pb_out, cfl, tsbits, dtb_dev);
    cudaError_t ce = cudaStreamEndCapture(st, &g);
    if (r != OM_OK) { if (g) cudaGraphDestroy(g); return r; }
    if (ce != cudaSuccess) {
      set_error(std::string("adjoint graph capture: ") + cudaGetErrorString(ce));
      return OM_ERR_CUDA;
    }
    ce = cudaGraphInstantiate(&s->graph[key], g, 0);
    cudaGraphDestroy(g);
    if (ce != cudaSuccess) {
      set_error(std::string("adjoint graph instantiate: ") + cudaGetErrorString(ce));
      return OM_ERR_CUDA;
    }
    s->graph_ub[key] = ub[0];
    std::memcpy(s->graph_scalars[key], baked, sizeof(baked));
  }
  OM_CUDA_CHECK(cudaGraphLaunch(s->graph[key], st));
  h->launches += 9;
  return OM_OK;
}

}  // namespace om

using namespace om;

extern "C" om_status om_hydro_vjp(om_handle H, void *const *cot_next, void *const *cot_prev) {
  Handle *h = handle_of(H);
  if (!h || h->kind != OM_KIND_HYDRO || !cot_next || !cot_prev) {
    set_error("om_hydro_vjp: needs a Hydro handle and 4 + 4 device arrays");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  const int fp64 = h->cfg.precision == 64;
  AdjointScratch *s;
  OM_TRY(get_scratch(h, fp64, &s));
  for (int i = 0; i < 4; ++i) OM_TRY(bring_device(h, h->arrays[i]));
  double dt;
  unsigned long long bits;
  OM_TRY(hydro_current_dt(h, &dt, &bits));
  void *state[4] = {h->arrays[0].d(), h->arrays[1].d(), h->arrays[2].d(), h->arrays[3].d()};
  const double cfl = ((HydroScalars *)h->h_scalars)->cfl;
  om_status st = fp64 ? vjp_kernels_direct<double>(h, s, state, cot_next, cot_prev, dt, cfl, bits)
                      : vjp_kernels_direct<float>(h, s, state, cot_next, cot_prev, dt, cfl, bits);
  OM_TRY(st);
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  return OM_OK;
}

// Gradient of loss = mean((density_T - target)^2) with respect to the state
// at the start, over `steps` proceed steps of the handle (which ends at
// step T).  sqrt(T) checkpointing: every s-th state is kept, each segment is
// recomputed once and walked backwards.
extern "C" om_status om_hydro_adjoint_run(om_handle H, int steps, const void *target,
                                          int checkpoint_every, double *loss,
                                          void *const *grad) {
  Handle *h = handle_of(H);
  if (!h || h->kind != OM_KIND_HYDRO || steps < 1 || !target || !grad) {
    set_error("om_hydro_adjoint_run: needs a Hydro handle, steps >= 1, target and 4 outputs");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  const int fp64 = h->cfg.precision == 64;
  const size_t cells = h->memory_size_total();
  const size_t bytes = cells * (fp64 ? 8 : 4);
  AdjointScratch *sc;
  OM_TRY(get_scratch(h, fp64, &sc));
  const int seg = checkpoint_every > 0 ? checkpoint_every
                                       : std::max(1, (int)std::ceil(std::sqrt((double)steps)));
  const int nck = (steps + seg - 1) / seg;
  int kid = -1;
  OM_TRY(om_kernel_id(H, "proceed", &kid));
  std::vector<HydroCheckpoint> ck(nck + 1), segst(seg);
  std::vector<double> seg_dt(seg);
  std::vector<unsigned long long> seg_bits(seg);
  void *dtarget = nullptr;
  om_status status = OM_OK;
  auto fail = [&](om_status s2) {
    for (auto &c : ck) hydro_checkpoint_free(&c);
    for (auto &c : segst) hydro_checkpoint_free(&c);
    cudaFree(dtarget);
    return s2;
  };
  for (auto &c : ck)
    if ((status = hydro_checkpoint_alloc(h, &c)) != OM_OK) return fail(status);
  for (auto &c : segst)
    if ((status = hydro_checkpoint_alloc(h, &c)) != OM_OK) return fail(status);
  if (cudaMalloc(&dtarget, bytes) != cudaSuccess) {
    cudaGetLastError();
    set_error("om_hydro_adjoint_run: allocation failed");
    return fail(OM_ERR_NOMEM);
  }
  if (cudaMemcpy(dtarget, target, bytes, cudaMemcpyDefault) != cudaSuccess) {
    set_error("om_hydro_adjoint_run: target copy failed");
    return fail(OM_ERR_CUDA);
  }
  // forward with checkpoints
  for (int j = 0; j < nck; ++j) {
    if ((status = hydro_save(h, &ck[j])) != OM_OK) return fail(status);
    const int len = std::min(seg, steps - j * seg);
    if ((status = om_run_n(H, kid, len)) != OM_OK) return fail(status);
  }
  if ((status = hydro_save(h, &ck[nck])) != OM_OK) return fail(status);
  // loss and its cotangent at the final state
  {
    const int grid = sc->nparts;
    if (fp64)
      adj::adj_loss<double><<<grid, 256, 0, h->stream>>>(
          (const double *)h->arrays[0].d(), (const double *)dtarget, (double *)sc->ub[0], cells,
          sc->partials);
    else
      adj::adj_loss<float><<<grid, 256, 0, h->stream>>>(
          (const float *)h->arrays[0].d(), (const float *)dtarget, (float *)sc->ub[0], cells,
          sc->partials);
    for (int k = 1; k < 4; ++k) cudaMemsetAsync(sc->ub[k], 0, bytes, h->stream);
    std::vector<double> part(grid);
    cudaMemcpyAsync(part.data(), sc->partials, sizeof(double) * grid, cudaMemcpyDeviceToHost,
                    h->stream);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
      set_error(std::string("adjoint loss: ") + cudaGetErrorString(cudaGetLastError()));
      return fail(OM_ERR_CUDA);
    }
    double l = 0;
    for (double v : part) l += v;
    if (loss) *loss = l / (double)cells;
  }
  // backward, segment by segment
  void *ub[4] = {sc->ub[0], sc->ub[1], sc->ub[2], sc->ub[3]};
  void *pb[4] = {sc->pb[0], sc->pb[1], sc->pb[2], sc->pb[3]};
  const double cfl = ((HydroScalars *)h->h_scalars)->cfl;
  for (int j = nck - 1; j >= 0; --j) {
    const int len = std::min(seg, steps - j * seg);
    if ((status = hydro_restore(h, &ck[j])) != OM_OK) return fail(status);
    for (int m = 0; m < len; ++m) {
      if ((status = hydro_save(h, &segst[m])) != OM_OK) return fail(status);
      if ((status = hydro_current_dt(h, &seg_dt[m], &seg_bits[m])) != OM_OK) return fail(status);
      if ((status = om_run(H, kid)) != OM_OK) return fail(status);
    }
    for (int m = len - 1; m >= 0; --m) {
      status = fp64 ? vjp_step<double>(h, sc, segst[m].f, ub, pb, &seg_dt[m], cfl, seg_bits[m],
                                       nullptr)
                    : vjp_step<float>(h, sc, segst[m].f, ub, pb, &seg_dt[m], cfl, seg_bits[m],
                                      nullptr);
      if (status != OM_OK) return fail(status);
      for (int k = 0; k < 4; ++k) std::swap(ub[k], pb[k]);
    }
  }
  for (int k = 0; k < 4; ++k)
    if (cudaMemcpyAsync(grad[k], ub[k], bytes, cudaMemcpyDefault, h->stream) != cudaSuccess) {
      set_error("om_hydro_adjoint_run: gradient copy failed");
      return fail(OM_ERR_CUDA);
    }
  // leave the handle at the final state of the forward run
  if ((status = hydro_restore(h, &ck[nck])) != OM_OK) return fail(status);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
    set_error(std::string("om_hydro_adjoint_run: ") + cudaGetErrorString(cudaGetLastError()));
    return fail(OM_ERR_CUDA);
  }
  return fail(OM_OK);
}

// device time (ms) of one adjoint step at the handle's current state, for
// measurement (cotangent input: the density cotangent of the loss)
extern "C" om_status om_hydro_time_vjp(om_handle H, int reps, float *ms) {
  Handle *h = handle_of(H);
  if (!h || h->kind != OM_KIND_HYDRO || reps < 1 || !ms) {
    set_error("om_hydro_time_vjp: bad arguments");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  const int fp64 = h->cfg.precision == 64;
  AdjointScratch *s;
  OM_TRY(get_scratch(h, fp64, &s));
  for (int i = 0; i < 4; ++i) OM_TRY(bring_device(h, h->arrays[i]));
  double dt;
  unsigned long long bits;
  OM_TRY(hydro_current_dt(h, &dt, &bits));
  const size_t bytes = h->memory_size_total() * (fp64 ? 8 : 4);
  for (int k = 0; k < 4; ++k) OM_CUDA_CHECK(cudaMemsetAsync(s->ub[k], 0, bytes, h->stream));
  void *state[4] = {h->arrays[0].d(), h->arrays[1].d(), h->arrays[2].d(), h->arrays[3].d()};
  const double cfl = ((HydroScalars *)h->h_scalars)->cfl;
  cudaEvent_t e0, e1;
  OM_CUDA_CHECK(cudaEventCreate(&e0));
  OM_CUDA_CHECK(cudaEventCreate(&e1));
  OM_CUDA_CHECK(cudaEventRecord(e0, h->stream));
  for (int r = 0; r < reps; ++r) {
    om_status st = fp64 ? vjp_step<double>(h, s, state, s->ub, s->pb, &dt, cfl, bits, nullptr)
                        : vjp_step<float>(h, s, state, s->ub, s->pb, &dt, cfl, bits, nullptr);
    OM_TRY(st);
  }
  OM_CUDA_CHECK(cudaEventRecord(e1, h->stream));
  OM_CUDA_CHECK(cudaEventSynchronize(e1));
  cudaEventElapsedTime(ms, e0, e1);
  *ms /= reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return OM_OK;
}

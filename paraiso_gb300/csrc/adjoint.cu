// adjoint.cu -- reverse-mode adjoint of the Hydro step on GB300 (no
// counterpart in the reference; the forward is examples/Hydro/HydroMain.hs
// proceed, HydroMain.hs:134-164).
//
// One adjoint step maps the cotangent of the state after a step to the
// cotangent of the state before it, through both stages, both axes, the
// MUSCL-minmod reconstruction, the HLLC fluxes, the clamps and the dt of the
// step (dt = cfl * min timescale: its cotangent is routed to the arg-min
// cell).  It reads the step's tape, written by the forward step itself when
// it is recomputed from a checkpoint (hydro_fused_tape_kernel: the stage-1
// state and both stages' flux differences), and runs as two launches over
// TX x TY tiles whose face work lives in shared memory, so every cotangent
// is written by exactly one thread, and one single-block launch:
//   B-D  stage-2 update reverse on the tile and a 2-cell halo, stage-2 walls
//        reverse (HLLC, MUSCL, per stencil slot in shared memory), gather
//        into the stage-1 cotangent, stage-1 update reverse; base part of the
//        previous-state cotangent, dt partial and minimum CFL timescale
//   E+F  stage-1 walls reverse and gather into the previous-state cotangent;
//        arg-min of the timescale
//   G    dt cotangent (partials summed in a fixed order) to the arg-min cell
// Multi-step gradients use sqrt(T) checkpointing: the forward keeps every
// s-th state; the backward recomputes each segment with the taped step and
// walks it backwards.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
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

// Indices reach at most a tile (32 x 16) plus 3 cells beyond the mesh; with
// both extents at least this, a single add or subtract wraps them.
constexpr int kCheapWrap = 40;

// What changes from one adjoint step to the next, read by the kernels from
// device memory so that one captured graph serves every step: where the
// step's CFL minimum is (its dt = cfl * minimum, formed in the OM's Real
// type as the forward step forms it), the four arrays of the state before
// the step and the step's tape.
struct StepIn {
  const unsigned long long *tsbits;  // CFL minimum of the state (hk::ts_bits)
  double cfl;
  void *state[4];
  // the step's tape: its arrays (hydro_kernels.cuh HydroTapeOut order:
  // q[4], d1[8], d2[8], u2[4]) lie `tape_pitch` bytes apart
  const void *tape;
  size_t tape_pitch;
  // the reverse step run just before this one (the step after it in time)
  // left its dt cotangent pending: it is added to this step's incoming
  // cotangent at that step's arg-min cell, whose state is prev_state
  int has_prev;
  void *prev_state[4];
};

// Where the pending dt cotangent of the previous reverse step is: its block
// partials (summed in a fixed order) and its arg-min cell.
struct PendingDt {
  const double *partials;
  int nparts;
  const unsigned long long *argmin;
};

// The taped arrays of a step: array k starts k * pitch elements after base.
// Array indices: stage-1 state 0..3, stage-1 differences 4..11, stage-2
// differences 12..19 (D[4 * axis + k]), stage-2 conserved state 20..23.
template <class R> struct TapeView {
  const R *base;
  size_t pitch;
  __device__ __forceinline__ const R *array(int k) const { return base + (size_t)k * pitch; }
  __device__ __forceinline__ void get8(int first, size_t i, R v[8]) const {
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = base[(size_t)(first + k) * pitch + i];
  }
  __device__ __forceinline__ Fields<R> fields(int first) const {
    return Fields<R>{{(R *)array(first), (R *)array(first + 1), (R *)array(first + 2),
                      (R *)array(first + 3)}};
  }
};
constexpr int kTapeQ = 0, kTapeD1 = 4, kTapeD2 = 12, kTapeU2 = 20;

template <class R> struct Geo {
  int n0, n1;
  R g, dR0, dR1, dt;
  const StepIn *in;   // this step's record (device memory)
  int cheap;          // n0, n1 >= kCheapWrap: one add or subtract wraps an index
  __device__ __forceinline__ R step_dt() const {
    return (R)in->cfl * hk::ts_from_bits<R>(*in->tsbits);
  }
  __device__ __forceinline__ Fields<R> state() const {
    return Fields<R>{{(R *)in->state[0], (R *)in->state[1], (R *)in->state[2],
                      (R *)in->state[3]}};
  }
  // the step's tape; read once per kernel (the record is in global memory,
  // so accesses through it after a store would be reloaded)
  __device__ __forceinline__ TapeView<R> tape() const {
    return TapeView<R>{(const R *)in->tape, in->tape_pitch / sizeof(R)};
  }
  // periodic index of a cell at most 4 cells (or one tile plus 3 cells)
  // outside the mesh
  __device__ __forceinline__ size_t at(int x, int y) const {
    if (cheap) {
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

// fixed-order sum of n doubles by a whole block: a strided sum per thread,
// then block_sum; every block that calls it gets the same bits
__device__ __forceinline__ double block_sum_of(const double *x, int n, double *sh);

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

__device__ __forceinline__ double block_sum_of(const double *x, int n, double *sh) {
  double acc = 0;
  for (int k = threadIdx.x; k < n; k += blockDim.x) acc += x[k];
  return block_sum(acc, sh);
}

// Tile shapes of the tile kernels
template <class R> struct AdjTile;
template <> struct AdjTile<float> { static constexpr int TX = 32, TY = 16; };
template <> struct AdjTile<double> { static constexpr int TX = 32, TY = 8; };

__device__ __forceinline__ unsigned long long warp_min(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
    v = w < v ? w : v;
  }
  return v;
}

// C+D on one TX x TY tile.  Stage-1 state box with a 3-cell halo (origin
// X0-3, Y0-3), stage-2 conserved-cotangent box with a 2-cell halo (origin
// X0-2, Y0-2), and per stencil slot the reconstruction cotangents of the
// faces whose stencils reach a tile cell: first the x faces X0-1 .. X0+TX+1
// of each tile row, then (in the same buffer) the y faces Y0-1 .. Y0+TY+1 of
// each tile column; the x part of the gather waits in qx.
template <class R, int TX, int TY> struct Stage2Smem {
  static constexpr int QX = TX + 6, QY = TY + 6;
  static constexpr int UX = TX + 4, UY = TY + 4;
  static constexpr int XF = TX + 3, YF = TY + 3;
  static constexpr int SLOTS = (TY * XF > YF * TX) ? TY * XF : YF * TX;
  R q[4][QY][QX];
  R u[4][UY][UX];
  R slot[16][SLOTS];  // [slot * 4 + field][face]; first the box inputs
  R qx[4][TY][TX];
  static_assert(8 * UY * UX <= 16 * SLOTS, "the box inputs are staged in the slot buffer");
};

template <class R> struct AdjOcc;  // CTAs per SM the tile kernels are built for
template <> struct AdjOcc<float> { static constexpr int stage2 = 3, stage1 = 4; };
template <> struct AdjOcc<double> { static constexpr int stage2 = 2, stage1 = 2; };

// Wait until the kernel launched before this one on the stream has finished
// and its writes are visible (a no-op unless this kernel was launched with
// programmatic stream serialization, when it may start while that one
// drains).
__device__ __forceinline__ void wait_previous_kernel() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
}

// 4- or 8-byte asynchronous copy global -> shared (cp.async, sm_80 and later)
template <class R>
__device__ __forceinline__ void cp_async(R *dst, const R *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if (sizeof(R) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// MUSCL reverse of the four fields of one face into its 16 slot values
template <class R>
__device__ __forceinline__ void face_slots(const Prim<R> st[4], const PrimBar<R> &Lb,
                                           const PrimBar<R> &Rb, R out[16]) {
  const R lb[4] = {Lb.rho, Lb.v0, Lb.v1, Lb.p}, rb[4] = {Rb.rho, Rb.v0, Rb.v1, Rb.p};
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    R xb[4] = {0, 0, 0, 0};
    ha::muscl_rev((&st[0].rho)[c], (&st[1].rho)[c], (&st[2].rho)[c], (&st[3].rho)[c], lb[c],
                  rb[c], xb[0], xb[1], xb[2], xb[3]);
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k * 4 + c] = xb[k];
  }
}

// HLLC and MUSCL reverse of one stage-2 face along AX: stencil st[4] (the
// stage-1 states of cells f-2 .. f+1), wall-flux cotangent fb -> 16 slots
template <int AX, class R>
__device__ __forceinline__ void face2_rev(const hf::Consts<R> &KC, const Prim<R> st[4],
                                          const Flux<R> &fb, R out[16]) {
  Prim<R> L, Rt;
  hs::muscl(st[0].rho, st[1].rho, st[2].rho, st[3].rho, L.rho, Rt.rho);
  hs::muscl(st[0].v0, st[1].v0, st[2].v0, st[3].v0, L.v0, Rt.v0);
  hs::muscl(st[0].v1, st[1].v1, st[2].v1, st[3].v1, L.v1, Rt.v1);
  hs::muscl(st[0].p, st[1].p, st[2].p, st[3].p, L.p, Rt.p);
  PrimBar<R> Lb, Rb;
  ha::zero(Lb);
  ha::zero(Rb);
  ha::hllc_rev<AX>(KC, L, Rt, fb, Lb, Rb);
  face_slots(st, Lb, Rb, out);
}

// C+D: stage-2 walls reverse (HLLC and MUSCL of the faces around the tile,
// cotangents kept per stencil slot in shared memory), then per tile cell the
// gather into Qb (face f = q + df holds the cell in slot 2 - df) and the
// stage-1 update reverse.
template <class R, int TX, int TY>
__global__ void __launch_bounds__(256, AdjOcc<R>::stage2)
adj_stage2_tile(Fields<R> Ub, Fields<R> U1b, Fields<R> Pbase, Geo<R> G, double *partial,
                unsigned long long *minbits, PendingDt pending) {
  using S = Stage2Smem<R, TX, TY>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S &s = *reinterpret_cast<S *>(smem_raw);
  __shared__ double sh[8];
  __shared__ unsigned long long pend_j;
  __shared__ R pend[4];
  wait_previous_kernel();
  G.dt = G.step_dt();
  const hf::Consts<R> KC = hf::consts<R>(G.g);
  const Fields<R> P = G.state();
  const TapeView<R> T = G.tape();
  const Fields<R> Q = T.fields(kTapeQ), U2 = T.fields(kTapeU2);
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int nt0 = (G.n0 + TX - 1) / TX;
  const int X0 = (int)(blockIdx.x % nt0) * TX, Y0 = (int)(blockIdx.x / nt0) * TY;
  // the stage-1 state box, and the stage-2 box's taped conserved state and
  // incoming cotangent (staged in the slot buffer, free until the faces),
  // copied asynchronously in one batch
  R(*stg)[S::UY][S::UX] = reinterpret_cast<R(*)[S::UY][S::UX]>(&s.slot[0][0]);
  for (int i = tid; i < S::QY * S::QX; i += nthr) {
    const int by = i / S::QX, bx = i - by * S::QX;
    const size_t gi = G.at(X0 - 3 + bx, Y0 - 3 + by);
#pragma unroll
    for (int c = 0; c < 4; ++c) cp_async(&s.q[c][by][bx], &Q.f[c][gi]);
  }
  for (int i = tid; i < S::UY * S::UX; i += nthr) {
    const int by = i / S::UX, bx = i - by * S::UX;
    const size_t gi = G.at(X0 - 2 + bx, Y0 - 2 + by);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      cp_async(&stg[c][by][bx], &U2.f[c][gi]);
      cp_async(&stg[4 + c][by][bx], &Ub.f[c][gi]);
    }
  }
  // the last phase reads the tile's taped flux differences of both stages
  // and its previous state per cell: bring their lines into L2 while the
  // earlier phases run
  {
    constexpr int kLine = 128 / (int)sizeof(R);           // elements per 128-byte line
    constexpr int LPR = (TX + kLine - 1) / kLine;         // lines per tile row
    for (int k = tid; k < 20 * TY * LPR; k += nthr) {
      const int arr = k / (TY * LPR), rem = k - arr * (TY * LPR);
      const int ry = rem / LPR, x = X0 + (rem - ry * LPR) * kLine, y = Y0 + ry;
      if (y >= G.n1 || x >= G.n0) continue;
      const R *base = arr < 16 ? T.array(kTapeD1 + arr) : P.f[arr - 16];
      asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (size_t)y * G.n0 + x));
    }
  }
  cp_async_wait_all();
  const R d0 = G.dt / G.dR0, d1 = G.dt / G.dR1;
  // the previous reverse step's dt cotangent, when its arg-min cell lies in
  // this tile's stage-2 box (blocks that find it compute the same value)
  if (tid == 0) {
    pend_j = ~0ull;
    if (G.in->has_prev) {
      const unsigned long long j = *pending.argmin;
      if (j != ~0ull) {
        const int jx = (int)(j % (unsigned long long)G.n0), jy = (int)(j / (unsigned long long)G.n0);
        const int dx = ((jx - (X0 - 2)) % G.n0 + G.n0) % G.n0;
        const int dy = ((jy - (Y0 - 2)) % G.n1 + G.n1) % G.n1;
        if (dx < S::UX && dy < S::UY) pend_j = j;
      }
    }
  }
  __syncthreads();
  if (pend_j != ~0ull) {
    const double dtb = block_sum_of(pending.partials, pending.nparts, sh);
    if (tid == 0) {
      const Fields<R> X{{(R *)G.in->prev_state[0], (R *)G.in->prev_state[1],
                         (R *)G.in->prev_state[2], (R *)G.in->prev_state[3]}};
      PrimBar<R> xb;
      ha::zero(xb);
      // dt = (Real)cfl * min: the minimum's cotangent is dt's times (Real)cfl
      const R cfl = (R)G.in->cfl;
      ha::timescale_rev(G.g, G.dR0, G.dR1, X.get(pend_j), (R)(dtb * (double)cfl), xb);
      pend[0] = xb.rho; pend[1] = xb.v0; pend[2] = xb.v1; pend[3] = xb.p;
    }
    __syncthreads();
  }
  // B: the stage-2 update reverse on the tile and a 2-cell halo, the
  // conserved cotangent of each cell's stage-2 update from the next-state
  // cotangent and the taped conserved state
  for (int i = tid; i < S::UY * S::UX; i += nthr) {
    const int by = i / S::UX, bx = i - by * S::UX;
    const size_t gi = G.at(X0 - 2 + bx, Y0 - 2 + by);
    const R u[4] = {stg[0][by][bx], stg[1][by][bx], stg[2][by][bx], stg[3][by][bx]};
    PrimBar<R> qb{stg[4][by][bx], stg[5][by][bx], stg[6][by][bx], stg[7][by][bx]};
    if (gi == pend_j) {
      qb.rho += pend[0]; qb.v0 += pend[1]; qb.v1 += pend[2]; qb.p += pend[3];
    }
    R U[4];
    ha::cons_from_prim_rev(G.g, u[0], u[1], u[2], u[3], qb, U);
#pragma unroll
    for (int c = 0; c < 4; ++c) s.u[c][by][bx] = U[c];
  }
  __syncthreads();
  // x faces: face X0-1+j of row Y0+r has stencil box columns j..j+3 of box
  // row r+3 and cells (right, left) at stage-2 cotangent box columns j+1, j of row r+2
  for (int i = tid; i < TY * S::XF; i += nthr) {
    const int r = i / S::XF, j = i - r * S::XF;
    Prim<R> st[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      st[k] = Prim<R>{s.q[0][r + 3][j + k], s.q[1][r + 3][j + k], s.q[2][r + 3][j + k],
                      s.q[3][r + 3][j + k]};
    const Flux<R> fb{d0 * (s.u[0][r + 2][j + 1] - s.u[0][r + 2][j]),
                     d0 * (s.u[1][r + 2][j + 1] - s.u[1][r + 2][j]),
                     d0 * (s.u[2][r + 2][j + 1] - s.u[2][r + 2][j]),
                     d0 * (s.u[3][r + 2][j + 1] - s.u[3][r + 2][j])};
    R out[16];
    face2_rev<0>(KC, st, fb, out);
#pragma unroll
    for (int k = 0; k < 16; ++k) s.slot[k][i] = out[k];
  }
  __syncthreads();
  for (int i = tid; i < TX * TY; i += nthr) {
    const int ty = i / TX, tx = i - ty * TX;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      R acc = R(0);
#pragma unroll
      for (int df = -1; df <= 2; ++df) acc += s.slot[(2 - df) * 4 + c][ty * S::XF + tx + df + 1];
      s.qx[c][ty][tx] = acc;
    }
  }
  __syncthreads();
  // y faces: face Y0-1+j of column X0+r has stencil box rows j..j+3 of box
  // column r+3 and cells at stage-2 cotangent box rows j+1, j of column r+2
  for (int i = tid; i < S::YF * TX; i += nthr) {
    const int j = i / TX, r = i - j * TX;
    Prim<R> st[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
      st[k] = Prim<R>{s.q[0][j + k][r + 3], s.q[1][j + k][r + 3], s.q[2][j + k][r + 3],
                      s.q[3][j + k][r + 3]};
    const Flux<R> fb{d1 * (s.u[0][j + 1][r + 2] - s.u[0][j][r + 2]),
                     d1 * (s.u[1][j + 1][r + 2] - s.u[1][j][r + 2]),
                     d1 * (s.u[2][j + 1][r + 2] - s.u[2][j][r + 2]),
                     d1 * (s.u[3][j + 1][r + 2] - s.u[3][j][r + 2])};
    R out[16];
    face2_rev<1>(KC, st, fb, out);
#pragma unroll
    for (int k = 0; k < 16; ++k) s.slot[k][i] = out[k];
  }
  __syncthreads();
  const R h = G.dt / R(2);
  const R e0 = h / G.dR0, e1 = h / G.dR1;
  const R rdR0 = R(1) / G.dR0, rdR1 = R(1) / G.dR1;
  double dtb = 0;
  unsigned long long best = ~0ull;
  for (int i = tid; i < TX * TY; i += nthr) {
    const int ty = i / TX, tx = i - ty * TX;
    const int x = X0 + tx, y = Y0 + ty;
    if (x >= G.n0 || y >= G.n1) continue;
    R qb[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      R acc = R(0);
#pragma unroll
      for (int df = -1; df <= 2; ++df) acc += s.slot[(2 - df) * 4 + c][(ty + df + 1) * TX + tx];
      qb[c] = s.qx[c][ty][tx] + acc;
    }
    const size_t gi = (size_t)y * G.n0 + x;
    R D[8];
    T.get8(kTapeD1, gi, D);
    const Prim<R> b = P.get(gi);
    R u[4];
    ha::update_cons_d(G.g, b, e0, e1, D, u);
    const PrimBar<R> qbar{qb[0], qb[1], qb[2], qb[3]};
    R U[4];
    ha::cons_from_prim_rev(G.g, u[0], u[1], u[2], u[3], qbar, U);
    U1b.set(gi, Prim<R>{U[0], U[1], U[2], U[3]});
    // base parts of both stages' updates (the stage-2 conserved cotangent
    // of this cell is the centre of the box)
    const R U2[4] = {s.u[0][ty + 2][tx + 2], s.u[1][ty + 2][tx + 2], s.u[2][ty + 2][tx + 2],
                     s.u[3][ty + 2][tx + 2]};
    PrimBar<R> bb;
    ha::zero(bb);
    ha::cons_of_prim_rev(G.g, b, U2, bb);
    ha::cons_of_prim_rev(G.g, b, U, bb);
    Pbase.set(gi, Prim<R>{bb.rho, bb.v0, bb.v1, bb.p});
    const R t0 = U[0] * D[0] + U[1] * D[1] + U[2] * D[2] + U[3] * D[3];
    const R t1 = U[0] * D[4] + U[1] * D[5] + U[2] * D[6] + U[3] * D[7];
    // dtdx = (dt / 2) / dR
    dtb += (double)(R(0.5) * (t0 * rdR0 + t1 * rdR1));
    T.get8(kTapeD2, gi, D);
    const R s0 = U2[0] * D[0] + U2[1] * D[1] + U2[2] * D[2] + U2[3] * D[3];
    const R s1 = U2[0] * D[4] + U2[1] * D[5] + U2[2] * D[6] + U2[3] * D[7];
    dtb += (double)(s0 * rdR0 + s1 * rdR1);
    const unsigned long long tb =
        hk::ts_bits<R>(hs::timescale(G.g, G.dR0, G.dR1, b.rho, b.v0, b.v1, b.p));
    best = tb < best ? tb : best;
  }
  best = warp_min(best);
  if ((tid & 31) == 0) atomicMin(minbits, best);
  const double sum = block_sum(dtb, sh);
  if (tid == 0) partial[blockIdx.x] = sum;
}

// E+F on one TX x TY tile (release: the other parity's arg-min slots, reset
// for the next step): the face cotangents (left-state part 0..3,
// right-state part 4..7) of x faces X0 .. X0+TX of each tile row and y faces
// Y0 .. Y0+TY of each tile column, then per tile cell the previous-state
// cotangent = base part + its own walls (right state) + the next walls
// (left state), and the lowest index whose CFL timescale equals the minimum
// (the arg-min that receives the dt cotangent; ties go to the lowest index).
template <class R, int TX, int TY> struct Stage1Smem {
  static constexpr int XF = TX + 1, YF = TY + 1, BX = TX + 2, BY = TY + 2;
  R fx[8][TY][XF];
  R fy[8][YF][TX];
  // the state (0..3) and the stage-1 cotangent (4..7) of cells X0-1 .. X0+TX,
  // Y0-1 .. Y0+TY
  R box[8][BY][BX];
};

template <class R, int TX, int TY>
__global__ void __launch_bounds__(256, AdjOcc<R>::stage1)
adj_stage1_tile(Fields<R> U1b, Fields<R> Pbase, Fields<R> Pb, Geo<R> G,
                const unsigned long long *minbits, unsigned long long *argmin,
                unsigned long long *release) {
  using S = Stage1Smem<R, TX, TY>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S &s = *reinterpret_cast<S *>(smem_raw);
  wait_previous_kernel();
  // the other parity's arg-min and minimum: read by this step's C+D kernel
  // (the pending dt of the step before), free now for the next step
  if (blockIdx.x == 0 && threadIdx.x == 0) release[0] = release[1] = ~0ull;
  G.dt = G.step_dt();
  const hf::Consts<R> KC = hf::consts<R>(G.g);
  const Fields<R> P = G.state();
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int nt0 = (G.n0 + TX - 1) / TX;
  const int X0 = (int)(blockIdx.x % nt0) * TX, Y0 = (int)(blockIdx.x / nt0) * TY;
  const R h = G.dt / R(2);
  const R d0 = h / G.dR0, d1 = h / G.dR1;
  // the box, copied asynchronously in one batch
  for (int i = tid; i < S::BY * S::BX; i += nthr) {
    const int by = i / S::BX, bx = i - by * S::BX;
    const size_t gi = G.at(X0 - 1 + bx, Y0 - 1 + by);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      cp_async(&s.box[c][by][bx], &P.f[c][gi]);
      cp_async(&s.box[4 + c][by][bx], &U1b.f[c][gi]);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  auto state = [&](int bx, int by) {
    return Prim<R>{s.box[0][by][bx], s.box[1][by][bx], s.box[2][by][bx], s.box[3][by][bx]};
  };
  auto cot = [&](int bx, int by) {
    return Prim<R>{s.box[4][by][bx], s.box[5][by][bx], s.box[6][by][bx], s.box[7][by][bx]};
  };
  constexpr int NXF = TY * S::XF, NYF = S::YF * TX;
  for (int i = tid; i < NXF + NYF; i += nthr) {
    PrimBar<R> Lb, Rb;
    ha::zero(Lb);
    ha::zero(Rb);
    int r, j;
    if (i < NXF) {
      // x face left of cell (X0 + j, Y0 + r): box cells (j + 1, r + 1), (j, r + 1)
      r = i / S::XF;
      j = i - r * S::XF;
      const Prim<R> a = cot(j + 1, r + 1), c = cot(j, r + 1);
      const Flux<R> fb{d0 * (a.rho - c.rho), d0 * (a.v0 - c.v0), d0 * (a.v1 - c.v1),
                       d0 * (a.p - c.p)};
      ha::hllc_rev<0>(KC, state(j, r + 1), state(j + 1, r + 1), fb, Lb, Rb);
      s.fx[0][r][j] = Lb.rho; s.fx[1][r][j] = Lb.v0; s.fx[2][r][j] = Lb.v1; s.fx[3][r][j] = Lb.p;
      s.fx[4][r][j] = Rb.rho; s.fx[5][r][j] = Rb.v0; s.fx[6][r][j] = Rb.v1; s.fx[7][r][j] = Rb.p;
    } else {
      // y face below cell (X0 + r, Y0 + j): box cells (r + 1, j + 1), (r + 1, j)
      const int i2 = i - NXF;
      j = i2 / TX;
      r = i2 - j * TX;
      const Prim<R> a = cot(r + 1, j + 1), c = cot(r + 1, j);
      const Flux<R> fb{d1 * (a.rho - c.rho), d1 * (a.v0 - c.v0), d1 * (a.v1 - c.v1),
                       d1 * (a.p - c.p)};
      ha::hllc_rev<1>(KC, state(r + 1, j), state(r + 1, j + 1), fb, Lb, Rb);
      s.fy[0][j][r] = Lb.rho; s.fy[1][j][r] = Lb.v0; s.fy[2][j][r] = Lb.v1; s.fy[3][j][r] = Lb.p;
      s.fy[4][j][r] = Rb.rho; s.fy[5][j][r] = Rb.v0; s.fy[6][j][r] = Rb.v1; s.fy[7][j][r] = Rb.p;
    }
  }
  __syncthreads();
  const unsigned long long mb = *minbits;
  unsigned long long best = ~0ull;
  for (int i = tid; i < TX * TY; i += nthr) {
    const int ty = i / TX, tx = i - ty * TX;
    const int x = X0 + tx, y = Y0 + ty;
    if (x >= G.n0 || y >= G.n1) continue;
    const size_t gi = (size_t)y * G.n0 + x;
    const Prim<R> q = state(tx + 1, ty + 1);
    if (hk::ts_bits<R>(hs::timescale(G.g, G.dR0, G.dR1, q.rho, q.v0, q.v1, q.p)) == mb &&
        gi < best)
      best = gi;
    Prim<R> b = Pbase.get(gi);
    b.rho += s.fx[4][ty][tx] + s.fx[0][ty][tx + 1] + s.fy[4][ty][tx] + s.fy[0][ty + 1][tx];
    b.v0 += s.fx[5][ty][tx] + s.fx[1][ty][tx + 1] + s.fy[5][ty][tx] + s.fy[1][ty + 1][tx];
    b.v1 += s.fx[6][ty][tx] + s.fx[2][ty][tx + 1] + s.fy[6][ty][tx] + s.fy[2][ty + 1][tx];
    b.p += s.fx[7][ty][tx] + s.fx[3][ty][tx + 1] + s.fy[7][ty][tx] + s.fy[3][ty + 1][tx];
    Pb.set(gi, b);
  }
  best = warp_min(best);
  if ((tid & 31) == 0 && best != ~0ull) atomicMin(argmin, best);
}

// G: dt cotangent of the last reverse step of a run to its arg-min cell
// (the others are applied by the next step's C+D kernel).  One block of 256
// threads sums the block partials in the fixed order of block_sum_of, as
// those kernels do; the arg-min cell's state and cotangent are fetched by
// the last warp while the others sum.
template <class R>
__global__ void __launch_bounds__(256)
adj_dt(Fields<R> Pb, Geo<R> G, const double *partials, int nparts, R cfl,
       const unsigned long long *argmin) {
  __shared__ double sh[8];
  __shared__ R cell[8];
  __shared__ unsigned long long jsh;
  if (threadIdx.x == blockDim.x - 32) {
    const unsigned long long j = *argmin;
    jsh = j;
    if (j != ~0ull) {
      const Prim<R> x = G.state().get(j), b = Pb.get(j);
      cell[0] = x.rho; cell[1] = x.v0; cell[2] = x.v1; cell[3] = x.p;
      cell[4] = b.rho; cell[5] = b.v0; cell[6] = b.v1; cell[7] = b.p;
    }
  }
  const double dtb = block_sum_of(partials, nparts, sh);
  if (threadIdx.x != 0) return;
  const unsigned long long j = jsh;
  if (j == ~0ull) return;
  const R tb = (R)(dtb * (double)cfl);
  PrimBar<R> xb;
  ha::zero(xb);
  ha::timescale_rev(G.g, G.dR0, G.dR1, Prim<R>{cell[0], cell[1], cell[2], cell[3]}, tb, xb);
  Pb.set(j, Prim<R>{cell[4] + xb.rho, cell[5] + xb.v0, cell[6] + xb.v1, cell[7] + xb.p});
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

// The tape of one step: HydroTapeOut's 24 arrays (q[4], d1[8], d2[8], u2[4])
// in one allocation, `pitch` bytes apart.
constexpr int kTapeArrays = 24;
struct StepTape {
  void *p[kTapeArrays] = {};
  size_t pitch = 0;
  HydroTapeOut out() const {
    HydroTapeOut t;
    for (int k = 0; k < 4; ++k) t.q[k] = p[k];
    for (int k = 0; k < 8; ++k) {
      t.d1[k] = p[4 + k];
      t.d2[k] = p[12 + k];
    }
    for (int k = 0; k < 4; ++k) t.u2[k] = p[20 + k];
    return t;
  }
};

// the arrays of a tape share one allocation (p[0] is its base)
static void tape_free(StepTape *t) {
  if (t->p[0]) cudaFree(t->p[0]);
  for (void *&q : t->p) q = nullptr;
}

static bool tape_alloc(size_t bytes, StepTape *t) {
  const size_t pitch = (bytes + 255) / 256 * 256;
  char *base = nullptr;
  if (cudaMalloc(&base, pitch * kTapeArrays) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  for (int k = 0; k < kTapeArrays; ++k) t->p[k] = base + pitch * k;
  t->pitch = pitch;
  return true;
}

struct AdjointScratch {
  int fp64 = -1;
  size_t cells = 0;
  void *u1b[4], *pbase[4], *ub[4], *pb[4], *next[4];
  StepTape tape1;                 // the tape of a single step
  HydroScalars *sc = nullptr;     // scalar block a single taped step updates
  double *dt_scratch = nullptr;
  adj::StepIn *d_in = nullptr;    // the record of a single step (device)
  adj::StepIn *h_in1 = nullptr;   // its pinned host copy
  // by step parity (the cotangent buffer a step reads): block partials of
  // the dt cotangent (ntiles each) and {arg-min cell, minimum bits}
  double *partials = nullptr;
  unsigned long long *argmin = nullptr;
  int nparts = 0;   // blocks of the grid-stride kernels
  int ntiles = 0;   // tiles of the reverse kernels (one dt partial each)
  std::vector<void *> all;
};

static void free_scratch(AdjointScratch *s) {
  if (!s) return;
  cudaFree(s->d_in);
  cudaFreeHost(s->h_in1);
  for (void *p : s->all) cudaFree(p);
  tape_free(&s->tape1);
  cudaFree(s->sc);
  cudaFree(s->dt_scratch);
  cudaFree(s->partials);
  cudaFree(s->argmin);
  delete s;
}

// scratch hangs off the handle through a small registry (handles of other
// threads may look it up at the same time)
static std::vector<std::pair<Handle *, AdjointScratch *>> g_scratch;
static std::mutex g_scratch_mu;

template <class R> static cudaError_t allow_tile_smem() {
  constexpr int TX = adj::AdjTile<R>::TX, TY = adj::AdjTile<R>::TY;
  const cudaError_t e = cudaFuncSetAttribute(adj::adj_stage2_tile<R, TX, TY>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sizeof(adj::Stage2Smem<R, TX, TY>));
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(adj::adj_stage1_tile<R, TX, TY>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(adj::Stage1Smem<R, TX, TY>));
}

static om_status get_scratch(Handle *h, int fp64, AdjointScratch **out) {
  if (!h->cyclic) {
    set_error("Hydro adjoint: periodic grids only");
    return OM_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  for (auto &kv : g_scratch)
    if (kv.first == h) {
      *out = kv.second;
      return OM_OK;
    }
  AdjointScratch *s = new AdjointScratch();
  s->fp64 = fp64;
  s->cells = h->memory_size_total();
  const size_t bytes = s->cells * (fp64 ? 8 : 4);
  void **groups[5] = {s->u1b, s->pbase, s->ub, s->pb, s->next};
  for (int gi = 0; gi < 5; ++gi)
    for (int k = 0; k < 4; ++k) {
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
  const int tx = fp64 ? adj::AdjTile<double>::TX : adj::AdjTile<float>::TX;
  const int ty = fp64 ? adj::AdjTile<double>::TY : adj::AdjTile<float>::TY;
  s->ntiles = ((h->size[0] + tx - 1) / tx) * ((h->size[1] + ty - 1) / ty);
  const cudaError_t ea = fp64 ? allow_tile_smem<double>() : allow_tile_smem<float>();
  if (ea != cudaSuccess || !tape_alloc(bytes, &s->tape1) ||
      cudaMalloc(&s->sc, sizeof(HydroScalars)) != cudaSuccess ||
      cudaMalloc(&s->dt_scratch, sizeof(double)) != cudaSuccess ||
      cudaMalloc(&s->partials, sizeof(double) * std::max(s->nparts, 2 * s->ntiles)) !=
          cudaSuccess ||
      cudaMalloc(&s->d_in, sizeof(adj::StepIn)) != cudaSuccess ||
      cudaMallocHost(&s->h_in1, sizeof(adj::StepIn)) != cudaSuccess ||
      cudaMalloc(&s->argmin, 4 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemset(s->argmin, 0xFF, 4 * sizeof(unsigned long long)) != cudaSuccess) {
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
  std::lock_guard<std::mutex> lock(g_scratch_mu);
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

// Launch of a kernel that may start while the previous kernel on the stream
// drains (programmatic stream serialization); the kernel waits for it with
// wait_previous_kernel before its first dependent read.
template <class... Params, class... Args>
static cudaError_t launch_after(void (*kernel)(Params...), int grid, size_t smem, cudaStream_t st,
                                Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(256);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, args...);
}

// both parities' arg-min slots to "none" (the start of a run)
static om_status reset_argmin(Handle *h, AdjointScratch *s) {
  OM_CUDA_CHECK(
      cudaMemsetAsync(s->argmin, 0xFF, 4 * sizeof(unsigned long long), h->stream));
  return OM_OK;
}

// kernels of one adjoint step, launched directly (the two tile kernels; the
// dt cotangent of a step is applied by the next step's first kernel, or by
// adj_dt after the last step of a run)
constexpr int kVjpLaunches = 2;

// The kernels of one adjoint step, reading the step's record `rec` (device
// memory): ub (4 device arrays, cotangent of the state after the step, less
// the previous reverse step's pending dt part) -> pb_out (4 device arrays,
// cotangent of the state before it, less this step's dt part, which is left
// pending in the parity-`par` partials and arg-min).  `par` is which of
// s->ub / s->pb the step reads.
template <class R>
static om_status vjp_kernels(Handle *h, AdjointScratch *s, const adj::StepIn *rec,
                             void *const *ub, void *const *pb_out, int par) {
  const cudaStream_t st = h->stream;
  const HydroScalars *hs_ = (const HydroScalars *)h->h_scalars;
  const int cheap = h->size[0] >= adj::kCheapWrap && h->size[1] >= adj::kCheapWrap;
  adj::Geo<R> G{h->size[0], h->size[1], (R)h->cfg.gamma, (R)hs_->dR0, (R)hs_->dR1, R(0), rec,
                cheap};
  const int nt = s->ntiles;
  constexpr int TX = adj::AdjTile<R>::TX, TY = adj::AdjTile<R>::TY;
  const auto U = F4<R>(ub), U1b = F4<R>(s->u1b), Pbase = F4<R>(s->pbase), Pb = F4<R>(pb_out);
  // argmin[2 par]: arg-min cell, argmin[2 par + 1]: minimum timescale bits
  unsigned long long *am = s->argmin + 2 * par;
  double *part = s->partials + (size_t)par * nt;
  unsigned long long *other = s->argmin + 2 * (1 - par);
  const adj::PendingDt pend{s->partials + (size_t)(1 - par) * nt, nt, other};
  // this parity's slots were reset by the previous step's E+F kernel (or by
  // reset_argmin at the start of the run)
  OM_CUDA_CHECK(launch_after(adj::adj_stage2_tile<R, TX, TY>, nt,
                             sizeof(adj::Stage2Smem<R, TX, TY>), st, U, U1b, Pbase, G, part,
                             am + 1, pend));
  OM_CUDA_CHECK(launch_after(adj::adj_stage1_tile<R, TX, TY>, nt,
                             sizeof(adj::Stage1Smem<R, TX, TY>), st, U1b, Pbase, Pb, G, am + 1,
                             am, other));
  h->launches += kVjpLaunches;
  return OM_OK;
}

static om_status run_vjp(Handle *h, AdjointScratch *s, const adj::StepIn *rec, void *const *ub,
                         void *const *pb) {
  const int par = ub[0] == s->ub[0] ? 0 : 1;
  return s->fp64 ? vjp_kernels<double>(h, s, rec, ub, pb, par)
                 : vjp_kernels<float>(h, s, rec, ub, pb, par);
}

// The dt cotangent left pending by the last reverse step of a run (parity
// par, record rec) added to its output pb.
template <class R>
static om_status final_dt(Handle *h, AdjointScratch *s, const adj::StepIn *rec,
                          void *const *pb, double cfl, int par) {
  const HydroScalars *hs_ = (const HydroScalars *)h->h_scalars;
  const int cheap = h->size[0] >= adj::kCheapWrap && h->size[1] >= adj::kCheapWrap;
  adj::Geo<R> G{h->size[0], h->size[1], (R)h->cfg.gamma, (R)hs_->dR0, (R)hs_->dR1, R(0), rec,
                cheap};
  adj::adj_dt<R><<<1, 256, 0, h->stream>>>(F4<R>(pb), G, s->partials + (size_t)par * s->ntiles,
                                           s->ntiles, (R)cfl, s->argmin + 2 * par);
  OM_CUDA_CHECK(cudaGetLastError());
  h->launches++;
  return OM_OK;
}

static om_status run_final_dt(Handle *h, AdjointScratch *s, const adj::StepIn *rec,
                              void *const *pb, double cfl, int par) {
  return s->fp64 ? final_dt<double>(h, s, rec, pb, cfl, par)
                 : final_dt<float>(h, s, rec, pb, cfl, par);
}

// One taped forward step between explicit buffers, in[4] -> out[4], with the
// adjoint's own scalar block s->sc: dt from s->sc->tsmin[read_slot], the CFL
// minimum of out into s->sc->tsmin[1 - read_slot].
static om_status launch_tape(Handle *h, AdjointScratch *s, void *const *in, void *const *out,
                             int read_slot, const HydroTapeOut &t) {
  HydroStepArgs a;
  a.rho = in[0]; a.v0 = in[1]; a.v1 = in[2]; a.p = in[3];
  a.nrho = out[0]; a.nv0 = out[1]; a.nv1 = out[2]; a.np = out[3];
  a.n0 = h->size[0]; a.n1 = h->size[1];
  a.nt0 = 0;
  a.gamma = h->cfg.gamma;
  a.gamma_f = (float)h->cfg.gamma;
  a.sc = s->sc;
  a.read_slot = read_slot;
  a.dt_hist = s->dt_scratch;
  a.lm = 0;
  a.ms0 = h->size[0];
  a.margin_min = nullptr;
  a.grid_limit = h->cfg.grid_limit;
  OM_CUDA_CHECK(cudaMemsetAsync(&s->sc->tsmin[1 - read_slot], 0xFF, sizeof(unsigned long long),
                                h->stream));
  const cudaError_t e = hydro_fused_tape(s->fp64, h->cfg.variant == 2, a, t, h->stream,
                                         hydro_tile_of(h->cfg.tile_x, h->cfg.tile_y,
                                                       !s->fp64 && h->cfg.variant == 0));
  if (e != cudaSuccess) {
    set_error(std::string("Hydro taped step: ") + cudaGetErrorString(e));
    return OM_ERR_CUDA;
  }
  h->launches++;
  return OM_OK;
}

// After a pass: a taped step whose bounded wait for its tensor copies ran
// out raised wait_error in the adjoint's scalar block (cleared here).
static om_status adjoint_waits(Handle *h, AdjointScratch *s) {
  uint32_t w = 0;
  OM_CUDA_CHECK(cudaMemcpyAsync(&w, &s->sc->wait_error, sizeof(w), cudaMemcpyDeviceToHost,
                                h->stream));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  if (!w) return OM_OK;
  OM_CUDA_CHECK(cudaMemsetAsync(&s->sc->wait_error, 0, sizeof(w), h->stream));
  set_error("Hydro adjoint: a taped step's bounded wait for its tensor copies ran out; the "
            "gradient of this pass is unspecified");
  return OM_ERR_CUDA;
}

// s->sc becomes a copy of the handle's scalar block with the CFL minimum of
// the handle's current state in tsmin[0].
static om_status load_scalars(Handle *h, AdjointScratch *s) {
  unsigned long long *ts = nullptr;
  OM_TRY(hydro_tsmin_device(h, &ts));
  OM_CUDA_CHECK(cudaMemcpyAsync(s->sc, h->d_scalars, sizeof(HydroScalars),
                                cudaMemcpyDeviceToDevice, h->stream));
  OM_CUDA_CHECK(cudaMemcpyAsync(&s->sc->tsmin[0], ts, sizeof(unsigned long long),
                                cudaMemcpyDeviceToDevice, h->stream));
  return OM_OK;
}

// The taped step of the handle's current state into s->tape1 (the handle
// does not move) and the record of that step in *in.
static om_status tape_current(Handle *h, AdjointScratch *s, adj::StepIn *in) {
  for (int k = 0; k < 4; ++k) OM_TRY(bring_device(h, h->arrays[k]));
  OM_TRY(load_scalars(h, s));
  void *cur[4];
  for (int k = 0; k < 4; ++k) cur[k] = h->arrays[k].d();
  OM_TRY(launch_tape(h, s, cur, s->next, 0, s->tape1.out()));
  in->tsbits = &s->sc->tsmin[0];
  in->cfl = ((HydroScalars *)h->h_scalars)->cfl;
  for (int k = 0; k < 4; ++k) in->state[k] = cur[k];
  in->tape = s->tape1.p[0];
  in->tape_pitch = s->tape1.pitch;
  in->has_prev = 0;
  for (int k = 0; k < 4; ++k) in->prev_state[k] = nullptr;
  return OM_OK;
}

}  // namespace om

using namespace om;

// The record of a checkpointed forward run, consumed by om_hydro_backward.
struct om_hydro_tape_s {
  Handle *h = nullptr;
  int steps = 0, seg = 0, nck = 0;
  std::vector<HydroCheckpoint> ck;     // state before segment j, and the final state
  std::vector<HydroCheckpoint> segst;  // states of one recomputed segment (1 .. seg-1)
  std::vector<StepTape> tapes;         // tapes of one recomputed segment (empty:
                                       // each step is taped again before its reverse)
  adj::StepIn *h_in = nullptr;         // pinned: one record per step
  adj::StepIn *d_recs = nullptr;       // the same, on the device (per segment)
  unsigned long long *d_ts = nullptr;  // CFL minimum of each step's state
  ~om_hydro_tape_s() {
    for (auto &c : ck) hydro_checkpoint_free(&c);
    for (auto &c : segst) hydro_checkpoint_free(&c);
    for (auto &t : tapes) tape_free(&t);
    if (h_in) cudaFreeHost(h_in);
    cudaFree(d_recs);
    cudaFree(d_ts);
  }
};

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
  // the pinned slot may still feed a step in flight
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  OM_TRY(tape_current(h, s, s->h_in1));
  const double cfl = ((HydroScalars *)h->h_scalars)->cfl;
  OM_CUDA_CHECK(cudaMemcpyAsync(s->d_in, s->h_in1, sizeof(adj::StepIn), cudaMemcpyHostToDevice,
                                h->stream));
  OM_TRY(reset_argmin(h, s));
  om_status st = fp64 ? vjp_kernels<double>(h, s, s->d_in, cot_next, cot_prev, 0)
                      : vjp_kernels<float>(h, s, s->d_in, cot_next, cot_prev, 0);
  OM_TRY(st);
  OM_TRY(run_final_dt(h, s, s->d_in, cot_prev, cfl, 0));
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  return OM_OK;
}

extern "C" om_status om_hydro_tape_free(om_hydro_tape tape) {
  delete tape;
  return OM_OK;
}

extern "C" om_status om_hydro_forward(om_handle H, int steps, int checkpoint_every,
                                      om_hydro_tape *out) {
  Handle *h = handle_of(H);
  if (!h || h->kind != OM_KIND_HYDRO || steps < 1 || !out) {
    set_error("om_hydro_forward: needs a Hydro handle, steps >= 1 and a tape pointer");
    return OM_ERR_ARG;
  }
  if (!h->cyclic) {
    set_error("Hydro adjoint: periodic grids only");
    return OM_ERR_UNSUPPORTED;
  }
  *out = nullptr;
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  om_hydro_tape t = new om_hydro_tape_s();
  t->h = h;
  t->steps = steps;
  t->seg = checkpoint_every > 0 ? checkpoint_every
                                : std::max(1, (int)std::ceil(std::sqrt((double)steps)));
  t->seg = std::min(t->seg, steps);
  t->nck = (steps + t->seg - 1) / t->seg;
  t->ck.resize(t->nck + 1);
  t->segst.resize(t->seg);
  om_status status = OM_OK;
  auto fail = [&](om_status s2) {
    delete t;
    return s2;
  };
  for (auto &c : t->ck)
    if ((status = hydro_checkpoint_alloc(h, &c)) != OM_OK) return fail(status);
  for (int m = 1; m < t->seg; ++m)  // a segment's first state is its checkpoint
    if ((status = hydro_checkpoint_alloc(h, &t->segst[m])) != OM_OK) return fail(status);
  {
    // one tape per step of a segment when they fit in half the free memory;
    // otherwise each step is taped again right before its reverse
    const size_t bytes = h->memory_size_total() * h->arrays[0].elem_size;
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
      cudaGetLastError();
      free_b = 0;
    }
    if ((double)bytes * kTapeArrays * t->seg <= 0.5 * (double)free_b &&
        !injected_alloc_failure()) {
      t->tapes.resize(t->seg);
      for (auto &tp : t->tapes)
        if (!tape_alloc(bytes, &tp)) {
          for (auto &q : t->tapes) tape_free(&q);
          t->tapes.clear();
          break;
        }
    }
  }
  if (cudaMallocHost(&t->h_in, sizeof(adj::StepIn) * (size_t)steps) != cudaSuccess ||
      cudaMalloc(&t->d_recs, sizeof(adj::StepIn) * (size_t)steps) != cudaSuccess ||
      cudaMalloc(&t->d_ts, sizeof(unsigned long long) * (size_t)steps) != cudaSuccess) {
    cudaGetLastError();
    set_error("om_hydro_forward: allocation failed");
    return fail(OM_ERR_NOMEM);
  }
  int kid = -1;
  if ((status = om_kernel_id(H, "proceed", &kid)) != OM_OK) return fail(status);
  for (int j = 0; j < t->nck; ++j) {
    if ((status = hydro_save(h, &t->ck[j])) != OM_OK) return fail(status);
    const int len = std::min(t->seg, steps - j * t->seg);
    if ((status = om_run_n(H, kid, len)) != OM_OK) return fail(status);
  }
  if ((status = hydro_save(h, &t->ck[t->nck])) != OM_OK) return fail(status);
  *out = t;
  return OM_OK;
}

// Backward over the tape from the final-state cotangent already in s->ub.
// On return result[4] holds the arrays (s->ub or s->pb) with the cotangent
// of the tape's start state; the handle is at the final state.  Each
// segment is recomputed from its checkpoint with the taped step, state to
// state on the device (no host round trip), keeping every step's CFL
// minimum, then walked backwards.  Every copy and kernel runs on the
// handle's stream, so a buffer is refilled only after the steps that read
// it.
static om_status backward_core(om_hydro_tape t, AdjointScratch *s, void **result) {
  Handle *h = t->h;
  void *ub[4], *pb[4];
  for (int k = 0; k < 4; ++k) {
    ub[k] = s->ub[k];
    pb[k] = s->pb[k];
  }
  const double cfl = ((HydroScalars *)h->h_scalars)->cfl;
  OM_TRY(reset_argmin(h, s));
  for (int j = t->nck - 1; j >= 0; --j) {
    const int len = std::min(t->seg, t->steps - j * t->seg);
    const bool taped = (int)t->tapes.size() >= len;
    OM_TRY(hydro_restore(h, &t->ck[j]));
    OM_TRY(load_scalars(h, s));
    for (int m = 0; m < len; ++m) {
      const int k = j * t->seg + m;
      adj::StepIn &in = t->h_in[k];
      void *const *cur = m == 0 ? t->ck[j].f : t->segst[m].f;
      void *const *nxt = m + 1 < len ? t->segst[m + 1].f : s->next;
      OM_CUDA_CHECK(cudaMemcpyAsync(&t->d_ts[k], &s->sc->tsmin[m & 1], sizeof(unsigned long long),
                                    cudaMemcpyDeviceToDevice, h->stream));
      in.tsbits = &t->d_ts[k];
      in.cfl = cfl;
      for (int q = 0; q < 4; ++q) in.state[q] = cur[q];
      const StepTape &tp = taped ? t->tapes[m] : s->tape1;
      in.tape = tp.p[0];
      in.tape_pitch = tp.pitch;
      // the step reversed before this one is the next in time: its state is
      // the next segment buffer, or the next segment's checkpoint; both stay
      // in place until this step has run
      in.has_prev = m + 1 < len || j + 1 < t->nck;
      for (int q = 0; q < 4; ++q)
        in.prev_state[q] = m + 1 < len ? t->segst[m + 1].f[q]
                                       : (j + 1 < t->nck ? t->ck[j + 1].f[q] : nullptr);
      OM_TRY(launch_tape(h, s, cur, nxt, m & 1, tp.out()));
    }
    // the segment's records, on the device for its reverse steps (the host
    // copies are not touched again in this pass)
    OM_CUDA_CHECK(cudaMemcpyAsync(t->d_recs + (size_t)j * t->seg, t->h_in + (size_t)j * t->seg,
                                  sizeof(adj::StepIn) * (size_t)len, cudaMemcpyHostToDevice,
                                  h->stream));
    for (int m = len - 1; m >= 0; --m) {
      const int k = j * t->seg + m;
      if (!taped) {
        // one tape buffer: tape this step again from its kept state
        const adj::StepIn &in = t->h_in[k];
        OM_CUDA_CHECK(cudaMemcpyAsync(&s->sc->tsmin[0], in.tsbits, sizeof(unsigned long long),
                                      cudaMemcpyDeviceToDevice, h->stream));
        OM_TRY(launch_tape(h, s, in.state, s->next, 0, s->tape1.out()));
      }
      OM_TRY(run_vjp(h, s, t->d_recs + k, ub, pb));
      for (int q = 0; q < 4; ++q) std::swap(ub[q], pb[q]);
    }
  }
  // the last step's dt cotangent (step 0; its parity: the buffer it read,
  // now pb)
  OM_TRY(run_final_dt(h, s, t->d_recs, ub, cfl, pb[0] == s->ub[0] ? 0 : 1));
  OM_TRY(hydro_restore(h, &t->ck[t->nck]));
  for (int k = 0; k < 4; ++k) result[k] = ub[k];
  return OM_OK;
}

extern "C" om_status om_hydro_backward(om_handle H, om_hydro_tape t, const void *const *cot_final,
                                       void *const *grad) {
  Handle *h = handle_of(H);
  if (!h || !t || t->h != h || !cot_final || !grad) {
    set_error("om_hydro_backward: needs the tape's own handle, 4 cotangents and 4 outputs");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  const int fp64 = h->cfg.precision == 64;
  const size_t bytes = h->memory_size_total() * (fp64 ? 8 : 4);
  AdjointScratch *s;
  OM_TRY(get_scratch(h, fp64, &s));
  for (int k = 0; k < 4; ++k)
    OM_CUDA_CHECK(cudaMemcpyAsync(s->ub[k], cot_final[k], bytes, cudaMemcpyDefault, h->stream));
  void *res[4];
  om_status status = backward_core(t, s, res);
  if (status != OM_OK) {
    hydro_restore(h, &t->ck[t->nck]);
    return status;
  }
  for (int k = 0; k < 4; ++k)
    OM_CUDA_CHECK(cudaMemcpyAsync(grad[k], res[k], bytes, cudaMemcpyDefault, h->stream));
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
    set_error(std::string("om_hydro_backward: ") + cudaGetErrorString(cudaGetLastError()));
    return OM_ERR_CUDA;
  }
  return adjoint_waits(h, s);
}

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
  void *dtarget = nullptr;
  if (cudaMalloc(&dtarget, bytes) != cudaSuccess) {
    cudaGetLastError();
    set_error("om_hydro_adjoint_run: allocation failed");
    return OM_ERR_NOMEM;
  }
  om_hydro_tape t = nullptr;
  auto done = [&](om_status s2) {
    if (t) om_hydro_tape_free(t);
    cudaFree(dtarget);
    return s2;
  };
  if (cudaMemcpy(dtarget, target, bytes, cudaMemcpyDefault) != cudaSuccess) {
    set_error("om_hydro_adjoint_run: target copy failed");
    return done(OM_ERR_CUDA);
  }
  om_status status = om_hydro_forward(H, steps, checkpoint_every, &t);
  if (status != OM_OK) return done(status);
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
      return done(OM_ERR_CUDA);
    }
    double l = 0;
    for (double v : part) l += v;
    if (loss) *loss = l / (double)cells;
  }
  void *res[4];
  if ((status = backward_core(t, sc, res)) != OM_OK) {
    hydro_restore(h, &t->ck[t->nck]);
    return done(status);
  }
  for (int k = 0; k < 4; ++k)
    if (cudaMemcpyAsync(grad[k], res[k], bytes, cudaMemcpyDefault, h->stream) != cudaSuccess) {
      set_error("om_hydro_adjoint_run: gradient copy failed");
      return done(OM_ERR_CUDA);
    }
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) {
    set_error(std::string("om_hydro_adjoint_run: ") + cudaGetErrorString(cudaGetLastError()));
    return done(OM_ERR_CUDA);
  }
  return done(adjoint_waits(h, sc));
}

// Device time (ms) of one adjoint step at the handle's current state, for
// measurement: the reverse sweep from the step's tape (made once, outside
// the timed region) with zero cotangents (the kernels' work does not depend
// on their values).
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
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  OM_TRY(tape_current(h, s, s->h_in1));
  const size_t bytes = h->memory_size_total() * (fp64 ? 8 : 4);
  for (int k = 0; k < 4; ++k) OM_CUDA_CHECK(cudaMemsetAsync(s->ub[k], 0, bytes, h->stream));
  // steps alternate the cotangent buffers as a backward pass does, each
  // applying the pending dt cotangent of the one before; two steps run
  // outside the timed region
  s->h_in1->has_prev = 1;
  for (int k = 0; k < 4; ++k) s->h_in1->prev_state[k] = s->h_in1->state[k];
  OM_CUDA_CHECK(cudaMemcpyAsync(s->d_in, s->h_in1, sizeof(adj::StepIn), cudaMemcpyHostToDevice,
                                h->stream));
  void *ub[4], *pb[4];
  for (int k = 0; k < 4; ++k) {
    ub[k] = s->ub[k];
    pb[k] = s->pb[k];
  }
  OM_TRY(reset_argmin(h, s));
  for (int r = 0; r < 2; ++r) {
    OM_TRY(run_vjp(h, s, s->d_in, ub, pb));
    for (int k = 0; k < 4; ++k) std::swap(ub[k], pb[k]);
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  om_status st = OM_OK;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
      cudaEventRecord(e0, h->stream) != cudaSuccess) {
    set_error("om_hydro_time_vjp: event setup failed");
    st = OM_ERR_CUDA;
  }
  for (int r = 0; st == OM_OK && r < reps; ++r) {
    st = run_vjp(h, s, s->d_in, ub, pb);
    for (int k = 0; k < 4; ++k) std::swap(ub[k], pb[k]);
  }
  if (st == OM_OK && (cudaEventRecord(e1, h->stream) != cudaSuccess ||
                      cudaEventSynchronize(e1) != cudaSuccess ||
                      cudaEventElapsedTime(ms, e0, e1) != cudaSuccess)) {
    set_error("om_hydro_time_vjp: timing failed");
    st = OM_ERR_CUDA;
  }
  if (st == OM_OK) *ms /= reps;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return st;
}

// Device time (ms) of one taped forward step at the handle's current state
// (the step the backward pass recomputes each segment with), mean of reps;
// the handle does not move.
extern "C" om_status om_hydro_time_tape(om_handle H, int reps, float *ms) {
  Handle *h = handle_of(H);
  if (!h || h->kind != OM_KIND_HYDRO || reps < 1 || !ms) {
    set_error("om_hydro_time_tape: bad arguments");
    return OM_ERR_ARG;
  }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  const int fp64 = h->cfg.precision == 64;
  AdjointScratch *s;
  OM_TRY(get_scratch(h, fp64, &s));
  adj::StepIn rec;
  OM_TRY(tape_current(h, s, &rec));  // warms up, and loads s->sc
  const HydroTapeOut out = s->tape1.out();
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  om_status st = OM_OK;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess ||
      cudaEventRecord(e0, h->stream) != cudaSuccess) {
    set_error("om_hydro_time_tape: event setup failed");
    st = OM_ERR_CUDA;
  }
  for (int r = 0; st == OM_OK && r < reps; ++r)
    st = launch_tape(h, s, rec.state, s->next, 0, out);
  if (st == OM_OK && (cudaEventRecord(e1, h->stream) != cudaSuccess ||
                      cudaEventSynchronize(e1) != cudaSuccess ||
                      cudaEventElapsedTime(ms, e0, e1) != cudaSuccess)) {
    set_error("om_hydro_time_tape: timing failed");
    st = OM_ERR_CUDA;
  }
  if (st == OM_OK) *ms /= reps;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  return st;
}

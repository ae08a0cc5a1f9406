// hydro_sweep.cuh -- the fused two-stage Hydro step as a column sweep.
//
// A block owns a strip of TX columns and a segment of rows and walks the
// segment downwards in chunks of TY rows.  The rows a chunk shares with the
// previous one stay in shared-memory rings: the primitive state and sound
// speeds (3 halo rows each side), the stage-1 cells (2 each side) and the
// stage-1 and stage-2 y walls (1 row).  So per chunk every quantity is
// computed for TY new rows only, and only the x halo (3 columns each side)
// is recomputed between neighbouring strips: about 4.3 HLLC evaluations per
// cell at TX = 32 (the minimum is 4: two walls per stage), where a 32 x 16
// tile with its full halo needs 5.0.  Each wall and cell is computed with
// exactly the operations of the tile kernel (hydro_kernels.cuh), so the two
// give the same results bit for bit in the exact builds.
//
// Scheme: examples/Hydro/HydroMain.hs:134-276 (proceed, proceedSingle,
// addFlux, interpolate, hllc); cyclic boundary only.
#pragma once

#include "hydro_kernels.cuh"

namespace om {

template <class R, int TX, int TY> struct SweepSmem {
  // ring capacities (rows): primitives and sound speeds are held as three
  // blocks of TY rows aligned to the segment's first box row (ya - 3): a
  // chunk reads two and the third is being loaded; stage-1 cells need the
  // chunk's rows and 2 halo rows each side, stage-1 y walls TY + 5 (the
  // first chunk of a segment computes them all), stage-2 y walls TY + 1
  static constexpr int RP = 3 * TY, RQ = TY + 4, RY1 = TY + 5, RY2 = TY + 1;
  static constexpr int PX = TX + 6, QX = TX + 4, X1 = TX + 5, X2 = TX + 1;
  R P[4][RP][PX];
  R C[RP][PX];
  R Q[4][RQ][QX];
  hs::Flux<R> s1y[RY1][QX];      // stage-1 walls between rows y-1 and y, columns X0-2 ..
  hs::Flux<R> s1x[TY + 4][X1];   // stage-1 x walls of this chunk's new stage-1 rows
  hs::Flux<R> s2y[RY2][TX];      // stage-2 walls between rows y-1 and y
  hs::Flux<R> s2x[TY][X2];       // stage-2 x walls of this chunk's rows
};

namespace sw {

// ring slot of row y (y >= -8)
template <int N> __device__ __forceinline__ int slot(int y) { return (y + 8 * N) % N; }

}  // namespace sw

// One strip (columns X0 .. X0+TX-1) over rows [ya, yb) of the grid of `a`,
// run by a whole block; the CFL minimum of the new state is folded into m.
template <class R, int TX, int TY, int NT, bool TAPE = false, bool FA = false>
__device__ __forceinline__ void sweep_segment(const HydroStepArgs &a, int X0, int ya, int yb,
                                              SweepSmem<R, TX, TY> &s, unsigned long long &m,
                                              const HydroTapeOut *tape = nullptr) {
  using S = SweepSmem<R, TX, TY>;
  const int tid = threadIdx.x;
  const int n0 = a.n0, n1 = a.n1;
  const R g = hk::Reals<R>::gamma(a);
  const hf::Consts<R> K = hf::consts<R>(g);
  const R dR0 = hk::Reals<R>::dR0(a.sc), dR1 = hk::Reals<R>::dR1(a.sc);
  const R dtG = hk::step_dt<R>(a);
  const R dtHalf = dtG / R(2);
  const R h0 = dtHalf / dR0, h1 = dtHalf / dR1;  // stage-1 dt/dR
  const R f0 = dtG / dR0, f1 = dtG / dR1;        // stage-2 dt/dR
  const R *rho = (const R *)a.rho, *vx = (const R *)a.v0, *vy = (const R *)a.v1,
          *pr = (const R *)a.p;
  R *orho = (R *)a.nrho, *ovx = (R *)a.nv0, *ovy = (R *)a.nv1, *opr = (R *)a.np;
  // box rows run from ya - 3 to below yb + 2 TY, columns from X0 - 3 to X0 + TX + 2
  const bool near = n0 >= TX + 8 && n1 >= 3 * TY + 8;
  // primitives: row y of the segment's box is ring row (y - ya + 3) mod RP;
  // block k is box rows ya - 3 + k TY .. + TY - 1, ring rows (k mod 3) TY ..
  auto load_block = [&](int k) {
    const int y0 = ya - 3 + k * TY;
    for (int i = tid; i < TY * S::PX; i += NT) {
      const int ry = i / S::PX, px = i - ry * S::PX;
      const int y = y0 + ry;
      const int gy = near ? hk::wrap_near(y, n1) : hk::wrap<R>(y, n1);
      const int gx = near ? hk::wrap_near(X0 + px - 3, n0) : hk::wrap<R>(X0 + px - 3, n0);
      const size_t gi = (size_t)gy * n0 + gx;
      const int sy = (k % 3) * TY + ry;
      hk::cp_async(&s.P[0][sy][px], rho + gi);
      hk::cp_async(&s.P[1][sy][px], vx + gi);
      hk::cp_async(&s.P[2][sy][px], vy + gi);
      hk::cp_async(&s.P[3][sy][px], pr + gi);
    }
    hk::cp_async_commit();
  };
  auto sound_block = [&](int k) {
    for (int i = tid; i < TY * S::PX; i += NT) {
      const int ry = i / S::PX, px = i - ry * S::PX;
      const int sy = (k % 3) * TY + ry;
      s.C[sy][px] = hk::face_sound<FA>(g, K, s.P[0][sy][px], s.P[3][sy][px]);
    }
  };
  auto pslot = [&](int y) { return (y - ya + 3) % S::RP; };
  for (int Ya = ya, c = 0; Ya < yb; Ya += TY, ++c) {
    const bool first = Ya == ya;
    // A: chunk c reads blocks c and c + 1 (box rows Ya - 3 .. Ya + TY + 2);
    // block c + 2 is loaded while the chunk computes (none after the last
    // chunk, so no copy is left in flight)
    if (first) {
      load_block(0);
      load_block(1);
    }
    hk::cp_async_wait_all();
    __syncthreads();
    if (first) sound_block(0);
    sound_block(c + 1);
    if (Ya + TY < yb) load_block(c + 2);
    __syncthreads();
    // B: stage-1 walls of the new stage-1 rows: x walls of rows q0 .., y
    // walls between rows y-1 and y for y in [w0, Ya + TY + 3)
    const int q0 = first ? Ya - 2 : Ya + 2, nq = first ? TY + 4 : TY;
    {
      const int w0 = first ? Ya - 2 : Ya + 3, nw = first ? TY + 5 : TY;
      constexpr int W1 = S::X1, W2 = S::QX;
      const int NX = nq * W1, NY = nw * W2;
      for (int i = tid; i < NX + NY; i += NT) {
        if (i < NX) {
          const int ry = i / W1, fx = i - ry * W1;  // wall between box columns fx, fx + 1
          const int sy = pslot(q0 + ry);
          const hs::Prim<R> L{s.P[0][sy][fx], s.P[1][sy][fx], s.P[2][sy][fx], s.P[3][sy][fx]};
          const hs::Prim<R> Rt{s.P[0][sy][fx + 1], s.P[1][sy][fx + 1], s.P[2][sy][fx + 1],
                               s.P[3][sy][fx + 1]};
          s.s1x[ry][fx] = hk::wall_flux<FA, 0>(g, K, L, s.C[sy][fx], Rt, s.C[sy][fx + 1]);
        } else {
          const int j = i - NX;
          const int ry = j / W2, cx = j - ry * W2;  // column X0 - 2 + cx
          const int y = w0 + ry;
          const int sa = pslot(y - 1), sb = pslot(y);
          const int px = cx + 1;
          const hs::Prim<R> L{s.P[0][sa][px], s.P[1][sa][px], s.P[2][sa][px], s.P[3][sa][px]};
          const hs::Prim<R> Rt{s.P[0][sb][px], s.P[1][sb][px], s.P[2][sb][px], s.P[3][sb][px]};
          s.s1y[sw::slot<S::RY1>(y)][cx] =
              hk::wall_flux<FA, 1>(g, K, L, s.C[sa][px], Rt, s.C[sb][px]);
        }
      }
    }
    __syncthreads();
    // C: the new stage-1 cells (rows q0 .., columns X0-2 .. X0+TX+1)
    for (int i = tid; i < nq * S::QX; i += NT) {
      const int ry = i / S::QX, qx = i - ry * S::QX;
      const int y = q0 + ry;
      const int sp = pslot(y), px = qx + 1;
      const hs::Prim<R> b{s.P[0][sp][px], s.P[1][sp][px], s.P[2][sp][px], s.P[3][sp][px]};
      const hs::Flux<R> &l0 = s.s1x[ry][qx], &r0 = s.s1x[ry][qx + 1];
      const hs::Flux<R> &l1 = s.s1y[sw::slot<S::RY1>(y)][qx];
      const hs::Flux<R> &r1 = s.s1y[sw::slot<S::RY1>(y + 1)][qx];
      const hs::Prim<R> q = hk::cell_update<FA>(g, K, b, h0, h1, l0, r0, l1, r1);
      const int sq = sw::slot<S::RQ>(y);
      s.Q[0][sq][qx] = q.rho;
      s.Q[1][sq][qx] = q.v0;
      s.Q[2][sq][qx] = q.v1;
      s.Q[3][sq][qx] = q.p;
      if (TAPE) {
        const int tx = qx - 2;
        if (tx >= 0 && tx < TX && y >= ya && y < yb && X0 + tx < n0) {
          const size_t gi = (size_t)y * n0 + (X0 + tx);
          ((R *)tape->q[0])[gi] = q.rho;
          ((R *)tape->q[1])[gi] = q.v0;
          ((R *)tape->q[2])[gi] = q.v1;
          ((R *)tape->q[3])[gi] = q.p;
          hk::tape_diffs<R>(tape->d1, gi, l0, r0, l1, r1);
        }
      }
    }
    __syncthreads();
    // D: stage-2 walls with MUSCL-minmod reconstruction of the stage-1
    // cells: x walls of the chunk's rows, y walls between rows y-1 and y for
    // y in [v0, Ya + TY + 1)
    {
      const int v0 = first ? Ya : Ya + 1, nv = first ? TY + 1 : TY;
      constexpr int W1 = S::X2, W2 = TX;
      constexpr int NX = TY * W1;
      const int NY = nv * W2;
      for (int i = tid; i < NX + NY; i += NT) {
        hs::Prim<R> L, Rt;
        if (i < NX) {
          const int ry = i / W1, sx = i - ry * W1;  // wall between columns X0-1+sx, X0+sx
          const int sq = sw::slot<S::RQ>(Ya + ry);
#pragma unroll
          for (int f = 0; f < 4; ++f) {
            R l, r;
            hk::muscl<FA>(s.Q[f][sq][sx], s.Q[f][sq][sx + 1], s.Q[f][sq][sx + 2],
                          s.Q[f][sq][sx + 3],
                      l, r);
            (&L.rho)[f] = l;
            (&Rt.rho)[f] = r;
          }
          s.s2x[ry][sx] = hk::wall_flux<FA, 0>(g, K, L, hk::face_sound<FA>(g, K, L.rho, L.p),
                                               Rt, hk::face_sound<FA>(g, K, Rt.rho, Rt.p));
        } else {
          const int j = i - NX;
          const int ry = j / W2, cx = j - ry * W2;
          const int y = v0 + ry, qx = cx + 2;
          const int a0 = sw::slot<S::RQ>(y - 2), a1 = sw::slot<S::RQ>(y - 1),
                    a2 = sw::slot<S::RQ>(y), a3 = sw::slot<S::RQ>(y + 1);
#pragma unroll
          for (int f = 0; f < 4; ++f) {
            R l, r;
            hk::muscl<FA>(s.Q[f][a0][qx], s.Q[f][a1][qx], s.Q[f][a2][qx], s.Q[f][a3][qx], l, r);
            (&L.rho)[f] = l;
            (&Rt.rho)[f] = r;
          }
          s.s2y[sw::slot<S::RY2>(y)][cx] = hk::wall_flux<FA, 1>(
              g, K, L, hk::face_sound<FA>(g, K, L.rho, L.p), Rt,
              hk::face_sound<FA>(g, K, Rt.rho, Rt.p));
        }
      }
    }
    __syncthreads();
    // E: the chunk's cells, written out, with the CFL minimum of the new state
    for (int i = tid; i < TY * TX; i += NT) {
      const int oy = i / TX, ox = i - oy * TX;
      const int gy = Ya + oy, gx = X0 + ox;
      if (gy >= yb || gx >= n0) continue;
      const int sp = pslot(gy), px = ox + 3;
      const hs::Prim<R> b{s.P[0][sp][px], s.P[1][sp][px], s.P[2][sp][px], s.P[3][sp][px]};
      const hs::Flux<R> &l0 = s.s2x[oy][ox], &r0 = s.s2x[oy][ox + 1];
      const hs::Flux<R> &l1 = s.s2y[sw::slot<S::RY2>(gy)][ox];
      const hs::Flux<R> &r1 = s.s2y[sw::slot<S::RY2>(gy + 1)][ox];
      R cons[4];
      const hs::Prim<R> q =
          hk::cell_update<FA>(g, K, b, f0, f1, l0, r0, l1, r1, TAPE ? cons : nullptr);
      const size_t gi = (size_t)gy * n0 + gx;
      if (TAPE) {
        hk::tape_diffs<R>(tape->d2, gi, l0, r0, l1, r1);
#pragma unroll
        for (int c = 0; c < 4; ++c) ((R *)tape->u2[c])[gi] = cons[c];
      }
      orho[gi] = q.rho;
      ovx[gi] = q.v0;
      ovy[gi] = q.v1;
      opr[gi] = q.p;
      const unsigned long long bits =
          hk::ts_bits<R>(hs::timescale(g, dR0, dR1, q.rho, q.v0, q.v1, q.p));
      m = bits < m ? bits : m;
    }
    // the next chunk's loads overwrite ring rows this chunk's last phase read
    __syncthreads();
  }
}

// the step's scalar bookkeeping, once per grid (by the block that owns the
// grid's first strip and segment): dt history, last dt, time
template <class R>
__device__ __forceinline__ void sweep_advance_time(const HydroStepArgs &a) {
  const R dtG = hk::step_dt<R>(a);
  a.dt_hist[0] = (double)dtG;
  a.sc->dt_last = (double)dtG;
  a.sc->time = a.sc->time + (double)dtG;
}

// Launch geometry of the sweep over an n0 x n1 grid: strips of TX columns,
// `segs` segments of `seg` rows (a multiple of TY; the last may be shorter).
struct SweepGeom {
  int strips, segs, seg;
};

// Segments per strip so that the blocks fill `resident` slots about four
// times over (the last wave stays short), each segment at least 4 chunks of
// TY rows.
inline SweepGeom sweep_geometry(int n0, int n1, int TX, int TY, int resident) {
  SweepGeom g;
  g.strips = (n0 + TX - 1) / TX;
  const int chunks = (n1 + TY - 1) / TY;
  int segs = 4 * resident / g.strips;
  if (segs < 1) segs = 1;
  if (segs > (chunks + 3) / 4) segs = (chunks + 3) / 4;
  if (segs < 1) segs = 1;
  const int cps = (chunks + segs - 1) / segs;  // chunks per segment
  g.seg = cps * TY;
  g.segs = (n1 + g.seg - 1) / g.seg;
  return g;
}

// One block per (strip, segment): blockIdx.x = segment * strips + strip.
template <class R, int TX, int TY, int NT, bool TAPE = false, bool FA = false>
__global__ void __launch_bounds__(NT)
hydro_sweep_kernel(HydroStepArgs a, SweepGeom geo, const __grid_constant__ HydroTapeOut t) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long red[32];
  auto &s = *reinterpret_cast<SweepSmem<R, TX, TY> *>(smem_raw);
  const int strip = blockIdx.x % geo.strips, seg = blockIdx.x / geo.strips;
  const int ya = seg * geo.seg, yb = min(a.n1, ya + geo.seg);
  unsigned long long m = ~0ull;
  sweep_segment<R, TX, TY, NT, TAPE, FA>(a, strip * TX, ya, yb, s, m, &t);
  hk::block_min_to(m, &a.sc->tsmin[1 - a.read_slot], red);
  if (blockIdx.x == 0 && threadIdx.x == 0) sweep_advance_time<R>(a);
}

}  // namespace om

// hydro_persist.cuh -- the persistent production FP32 step on 32 x 32
// tiles: the fused two-stage MUSCL-HLLC step of hydro_kernels.cuh
// (HydroMain.hs:169-276), in the production algebra (hf::), organised for
// the issue rate of a GB300 SM.
//
//  * A CTA strides over the tiles (single grid) or over the (instance,
//    tile) work list (ensembles).  While it computes one tile, the next
//    tile's 40 x 38 box of the four primitive fields lands in the other of
//    two box buffers: by TMA (four 2-D boxes completing on an mbarrier) for
//    tiles whose box lies inside the grid, by 16-byte cp.async with
//    periodically wrapped addresses for the edge tiles.
//  * The box is kept as four planes of 40 floats per row, starting 4 cells
//    left of the tile (a 16-byte aligned x coordinate) and 3 rows below it.
//  * Lanes run along rows of 32 walls or cells, so shared-memory accesses of
//    a warp are consecutive; the few walls and cells beyond 32 per row form
//    a short remainder list.
//  * The stage-1 state is kept as one float4 record per cell, in rows of 37
//    records (an odd pitch: a warp reading a column of records touches
//    every bank group once).
//  * Stage-2 walls are evaluated in runs of three consecutive walls along
//    the wall normal: the limited slope of a cell is formed once for the
//    right state of one wall and the left state of the next.  The 33 walls
//    of a row (or column) are 11 runs, so the 704 wall runs of a tile are
//    exactly one per thread of the 704-thread CTA.
//  * The paired form (PAIR, 352 threads) evaluates two walls or two cells
//    per thread with packed f32x2 instructions (hf::f2): a wall and the
//    wall 1344 items later, a cell and the cell 672 (stage 1) or 512
//    (stage 2) later (whole warps, so both halves of a warp run along
//    rows), a row's x-wall run with a column's y-wall run.  Walls of either
//    axis share the arithmetic in the frame of the wall; an item without a
//    partner is paired with itself and stored once.
//  * On large grids the paired form runs as one CTA per SM of two groups
//    (persist_run's GROUPS), each with its own shared-memory block and
//    named barrier, whose phases are offset by about half a tile.
//  * Stage 2 of a tile shares its pass with the next tile's sound speeds.
//  * The tile's CFL minimum is folded in registers over all the tiles of a
//    CTA or group (of one instance) and published once.
// Every value is formed by the production algebra's explicit operations
// (hf:: in hydro_scheme.cuh), as in the tile kernels of hydro_kernels.cuh,
// so all of them give the same bits.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "hydro_kernels.cuh"
#include "tma.cuh"

namespace om {
namespace hp {

constexpr int TX = 32, TY = 32;
constexpr int NT = 704;                 // 22 warps; two CTAs per SM
constexpr int NT2 = 352;                // the paired form: 11 warps; two CTAs (or groups) per SM
constexpr int BW = 40, BH = 38;         // box columns X0-4 .. X0+35, rows Y0-3 .. Y0+34
constexpr int PLANE = 1536;             // floats per field plane: 38 x 40 = 1520, padded to 6144 B
constexpr int QP = 37;                  // stage-1 records per row (36 used)
constexpr int F1X = 37, F1Y = 36;       // stage-1 walls per row: x walls (36 rows), y walls (37 rows)
constexpr int F2X = 33, F2Y = 32;       // stage-2 walls per row: x walls (32 rows), y walls (33 rows)
constexpr uint32_t kBoxBytes = 4u * BH * BW * 4u;  // bytes the four TMA boxes deliver

// stage-1 walls: rows of 32 walls first (x, then y), then the remainders
constexpr int kS1XMain = 36 * 32, kS1YMain = 37 * 32, kS1XRem = 36 * 5, kS1YRem = 37 * 4;
constexpr int kS1Items = kS1XMain + kS1YMain + kS1XRem + kS1YRem;  // 2664
constexpr int kQMain = 36 * 32, kQItems = 36 * 36;                  // stage-1 cells
// the paired form's second items start a whole number of warps later, so a
// warp's second items begin a row as its first ones do: wall i pairs with
// wall i + kS1Half (when that exists), cell i with cell i + kQHalf
constexpr int kS1Half = (kS1Items / 2 + 31) / 32 * 32;  // 1344
constexpr int kQHalf = (kQItems / 2 + 31) / 32 * 32;    // 672

using Flux = hs::Flux<float>;
using Prim = hs::Prim<float>;

struct alignas(128) Smem {
  float box[2][4 * PLANE];  // two boxes: planes rho, v0, v1, p (128-byte aligned)
  union {
    float c[BH * BW];     // sound speeds of the box cells (stage 1)
    float4 q[36 * QP];    // stage-1 state of the 36 x 36 cells (stage 2)
  } cq;
  union {
    struct {
      Flux x[36 * F1X];
      Flux y[37 * F1Y];
    } s1;
    struct {
      Flux x[32 * F2X];
      Flux y[33 * F2Y];
    } s2;
  } fl;
  uint64_t bar[2];
  uint64_t go;  // two groups per CTA: group 0 releases group 1 (in group 0's block)
  unsigned long long red[32];
  // ensembles: the arguments of the current and the next item's instance
  // (read from shared memory rather than held in registers across phases)
  HydroStepArgs args[2];
};

// two CTAs per SM, or one CTA of two groups, within the SM's shared memory
// (227 KB per CTA at most)
static_assert(2 * sizeof(Smem) <= 232448, "two shared-memory blocks per SM");

// a warp copies an argument block into shared memory
__device__ __forceinline__ void copy_args(HydroStepArgs *dst, const HydroStepArgs *src,
                                          int lane) {
  static_assert(sizeof(HydroStepArgs) % 4 == 0, "argument block of whole words");
  const uint32_t *s = reinterpret_cast<const uint32_t *>(src);
  uint32_t *d = reinterpret_cast<uint32_t *>(dst);
  for (int i = lane; i < (int)(sizeof(HydroStepArgs) / 4); i += 32) d[i] = s[i];
}

// a box lies inside the grid (no periodic image needed)
__device__ __forceinline__ bool box_inside(int X0, int Y0, int n0, int n1) {
  return X0 >= 4 && Y0 >= 3 && X0 + 36 <= n0 && Y0 + 35 <= n1;
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

// Start the copy of a tile's box into `dst`.  Inside the grid: thread 0
// posts the byte count on *bar and issues the four TMA boxes (maps[k]
// describes field k of this grid).  Else every thread copies 16-byte
// chunks with wrapped coordinates (grid sizes are multiples of 32, so a
// wrapped chunk stays 16-byte aligned).
// The four fields of a grid: their tensor maps (m, for boxes inside the
// grid) and base pointers (f).
struct FieldRefs {
  const CUtensorMap *m0, *m1, *m2, *m3;
  const float *f0, *f1, *f2, *f3;
};

template <int NTH = NT>
__device__ __forceinline__ void issue_box(float *dst, bool inside, const FieldRefs &r, int n0,
                                          int n1, int X0, int Y0, uint64_t *bar, int tid) {
  if (inside) {
    if (tid == 0) {
      tma::fence_proxy_async();
      tma::mbar_arrive_expect_tx(bar, kBoxBytes);
      tma::load_2d(dst, r.m0, X0 - 4, Y0 - 3, bar);
      tma::load_2d(dst + PLANE, r.m1, X0 - 4, Y0 - 3, bar);
      tma::load_2d(dst + 2 * PLANE, r.m2, X0 - 4, Y0 - 3, bar);
      tma::load_2d(dst + 3 * PLANE, r.m3, X0 - 4, Y0 - 3, bar);
    }
  } else {
    for (int i = tid; i < BH * 10; i += NTH) {
      const int py = i / 10, j = i - py * 10;
      const int gy = hk::wrap_near(Y0 - 3 + py, n1), gx = hk::wrap_near(X0 - 4 + 4 * j, n0);
      const size_t gi = (size_t)gy * n0 + gx;
      float *d = dst + py * BW + 4 * j;
      cp_async16(d, r.f0 + gi);
      cp_async16(d + PLANE, r.f1 + gi);
      cp_async16(d + 2 * PLANE, r.f2 + gi);
      cp_async16(d + 3 * PLANE, r.f3 + gi);
    }
    hk::cp_async_commit();
  }
}

__device__ __forceinline__ Prim box_cell(const float *B, int c) {
  return Prim{B[c], B[PLANE + c], B[2 * PLANE + c], B[3 * PLANE + c]};
}

__device__ __forceinline__ Prim rec(const float4 v) { return Prim{v.x, v.y, v.z, v.w}; }

// Three stage-2 walls along axis AX: wall j lies between records
// q[base + (j+1) st] and q[base + (j+2) st] and reconstructs from
// q[base + j st .. base + (j+3) st] (hf::muscl); its flux goes to
// out[j * ost].  The slope of the record right of wall j serves the left
// state of wall j+1.
template <int AX>
__device__ __forceinline__ void wall_run(const float4 *q, int base, int st, Flux *out, int ost,
                                         float g, const hf::Consts<float> &K) {
  Prim L;
  {
    const Prim x0 = rec(q[base]), x1 = rec(q[base + st]), x2 = rec(q[base + 2 * st]);
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const float a = (&x0.rho)[f], b = (&x1.rho)[f], c = (&x2.rho)[f];
      (&L.rho)[f] = hf::fma(hf::minmod(hf::sub(b, a), hf::sub(c, b)), 0.5f, b);
    }
  }
  float cl = hf::sound(K, L.rho, L.p);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const Prim x1 = rec(q[base + (j + 1) * st]), x2 = rec(q[base + (j + 2) * st]),
               x3 = rec(q[base + (j + 3) * st]);
    Prim R, Ln;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const float b = (&x1.rho)[f], c = (&x2.rho)[f], d = (&x3.rho)[f];
      const float s = hf::minmod(hf::sub(c, b), hf::sub(d, c));
      (&R.rho)[f] = hf::fma(s, -0.5f, c);
      (&Ln.rho)[f] = hf::fma(s, 0.5f, c);
    }
    const float cr = hf::sound(K, R.rho, R.p);
    out[j * ost] = hf::hllc<AX>(K, L, cl, R, cr);
    if (j < 2) {
      L = Ln;
      cl = hf::sound(K, L.rho, L.p);
    }
  }
}

// ---------------------------------------------------------------------------
// item maps shared by both forms
// ---------------------------------------------------------------------------

// stage-1 wall item i: axis, box index of the cell left of (below) the wall,
// and the wall's index in s1.x (axis 0) or s1.y (axis 1).  The wall joins
// box cells c and c + 1 (x) or c and c + BW (y).
__device__ __forceinline__ void s1_item(int i, int &ax, int &c, int &w) {
  int fy, fx;
  if (i < kS1XMain) {
    ax = 0; fy = i >> 5; fx = i & 31;
  } else if (i < kS1XMain + kS1YMain) {
    const int j = i - kS1XMain;
    ax = 1; fy = j >> 5; fx = j & 31;
  } else if (i < kS1XMain + kS1YMain + kS1XRem) {
    const int j = i - (kS1XMain + kS1YMain);
    ax = 0; fy = j / 5; fx = 32 + (j - fy * 5);
  } else {
    const int j = i - (kS1XMain + kS1YMain + kS1XRem);
    ax = 1; fy = j >> 2; fx = 32 + (j & 3);
  }
  // x wall fx of row fy: box cells (fy+1, fx+1), (fy+1, fx+2); y wall fx
  // of row fy: (fy, fx+2), (fy+1, fx+2)
  c = ax == 0 ? (fy + 1) * BW + fx + 1 : fy * BW + fx + 2;
  w = ax == 0 ? fy * F1X + fx : fy * F1Y + fx;
}

// stage-1 cell item i: (qy, qx) of the 36 x 36 cells
__device__ __forceinline__ void q_item(int i, int &qy, int &qx) {
  if (i < kQMain) {
    qy = i >> 5; qx = i & 31;
  } else {
    const int j = i - kQMain;
    qy = j >> 2; qx = 32 + (j & 3);
  }
}

// ---------------------------------------------------------------------------
// the paired form's helpers
// ---------------------------------------------------------------------------
using hf::f2;

__device__ __forceinline__ hf::NF<f2> pack_flux(const Flux &a, const Flux &b) {
  return hf::NF<f2>{hf::pack(a.fd, b.fd), hf::pack(a.fm0, b.fm0), hf::pack(a.fm1, b.fm1),
                    hf::pack(a.fe, b.fe)};
}

// a wall's flux from the frame of the wall back to axis order
__device__ __forceinline__ Flux axis_order(float fd, float fn, float ft, float fe, int ax) {
  Flux o;
  o.fd = fd;
  o.fm0 = ax == 0 ? fn : ft;
  o.fm1 = ax == 0 ? ft : fn;
  o.fe = fe;
  return o;
}

__device__ __forceinline__ void store_pair(const hf::NF<f2> &f, Flux *da, int axa, Flux *db,
                                           int axb) {
  float d0, d1, n0, n1, t0, t1, e0, e1;
  hf::unpack(f.fd, d0, d1);
  hf::unpack(f.fn, n0, n1);
  hf::unpack(f.ft, t0, t1);
  hf::unpack(f.fe, e0, e1);
  *da = axis_order(d0, n0, t0, e0, axa);
  *db = axis_order(d1, n1, t1, e1, axb);
}

// a box cell of wall a and one of wall b in the frames of their walls
__device__ __forceinline__ hf::NS<f2> pair_state(const float *B, int ca, int axa, int cb,
                                                 int axb) {
  const float va0 = B[PLANE + ca], va1 = B[2 * PLANE + ca];
  const float vb0 = B[PLANE + cb], vb1 = B[2 * PLANE + cb];
  return hf::NS<f2>{hf::pack(B[ca], B[cb]), hf::pack(axa == 0 ? va0 : va1, axb == 0 ? vb0 : vb1),
                    hf::pack(axa == 0 ? va1 : va0, axb == 0 ? vb1 : vb0),
                    hf::pack(B[3 * PLANE + ca], B[3 * PLANE + cb])};
}


// record k of the x run (row) and of the y run (column), in their walls'
// frames: (rho, un, ut, p)
__device__ __forceinline__ hf::NS<f2> run_rec(const float4 *q, int xa, int ya) {
  const float4 a = q[xa], b = q[ya];
  return hf::NS<f2>{hf::pack(a.x, b.x), hf::pack(a.y, b.z), hf::pack(a.z, b.y),
                    hf::pack(a.w, b.w)};
}

// The x-wall run of row `lane` (walls 3t..3t+2, records xb + 0..5) and the
// y-wall run of column `lane` (walls 3t..3t+2, records yb + 0..5 QP) side
// by side, as wall_run does for one run.
__device__ __forceinline__ void wall_run2(const float4 *q, int xb, int yb, Flux *xo, Flux *yo,
                                          const hf::K<f2> &k) {
  hf::NS<f2> L;
  {
    const hf::NS<f2> x0 = run_rec(q, xb, yb), x1 = run_rec(q, xb + 1, yb + QP),
                     x2 = run_rec(q, xb + 2, yb + 2 * QP);
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const f2 a = (&x0.rho)[f], b = (&x1.rho)[f], c = (&x2.rho)[f];
      (&L.rho)[f] = hf::fma(hf::minmod(hf::sub(b, a), hf::sub(c, b)), k.half, b);
    }
  }
  f2 cl = hf::sound(k, L.rho, L.p);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const hf::NS<f2> x1 = run_rec(q, xb + j + 1, yb + (j + 1) * QP),
                     x2 = run_rec(q, xb + j + 2, yb + (j + 2) * QP),
                     x3 = run_rec(q, xb + j + 3, yb + (j + 3) * QP);
    hf::NS<f2> R, Ln;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const f2 b = (&x1.rho)[f], c = (&x2.rho)[f], d = (&x3.rho)[f];
      const f2 sl = hf::minmod(hf::sub(c, b), hf::sub(d, c));
      (&R.rho)[f] = hf::fma(sl, k.neghalf, c);
      (&Ln.rho)[f] = hf::fma(sl, k.half, c);
    }
    const f2 cr = hf::sound(k, R.rho, R.p);
    store_pair(hf::hllc_ns<f2>(k, L, cl, R, cr), &xo[j], 0, &yo[j * F2Y], 1);
    if (j < 2) {
      L = Ln;
      cl = hf::sound(k, L.rho, L.p);
    }
  }
}

// ---------------------------------------------------------------------------
// the tile loop
// ---------------------------------------------------------------------------

// The tiles of one grid (ENS false: args[0], maps m[0..3]) or of an
// ensemble (ENS true: instance k has args[k], maps table[(k * 4) + field]
// and items pf[k] .. pf[k+1]-1).  TAPE: the taped step (single grid).
// PAIR: the paired form (NT2 threads), else one wall or cell per thread
// (NT threads).
// GROUPS 2: the CTA holds two independent groups of NTH threads, each with
// its own shared-memory block (sm[0], sm[1]) and named barrier, working on
// alternate items; group 1 starts once group 0 has passed the second phase
// of its first tile, so the two groups' phases run about half a tile apart
// and one group's barrier tails overlap the other's arithmetic.
template <bool TAPE, bool ENS, bool PAIR, int GROUPS = 1>
__device__ __forceinline__ void persist_run(const HydroStepArgs *__restrict__ args,
                                            const int *__restrict__ pf, int count,
                                            const CUtensorMap *table, const CUtensorMap *m0,
                                            const CUtensorMap *m1, const CUtensorMap *m2,
                                            const CUtensorMap *m3, Smem *sm,
                                            const HydroTapeOut *tape) {
  constexpr int NTH = PAIR ? NT2 : NT;
  const int grp = GROUPS == 2 ? (int)threadIdx.x / NTH : 0;
  Smem &s = sm[grp];
  const int tid = (int)threadIdx.x - grp * NTH, lane = tid & 31, warp = tid >> 5;
  auto sync = [&]() {
    if (GROUPS == 1) __syncthreads();
    else asm volatile("bar.sync %0, %1;" ::"r"(1 + grp), "r"(NTH) : "memory");
  };
  // block-wide (group-wide) min of CFL bit patterns folded into *dst
  auto min_to = [&](unsigned long long v, unsigned long long *dst) {
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
      v = w < v ? w : v;
    }
    if (lane == 0) s.red[warp] = v;
    sync();
    if (warp == 0) {
      v = lane < NTH / 32 ? s.red[lane] : ~0ull;
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w < v ? w : v;
      }
      if (lane == 0) atomicMin(dst, v);
    }
  };
  const int total =
      ENS ? pf[count] : args[0].nt0 * ((args[0].n1 + TY - 1) / TY);
  int item = (int)blockIdx.x * GROUPS + grp;
  const int stride = (int)gridDim.x * GROUPS;
  if (tid == 0) {
    tma::mbar_init(&s.bar[0], 1);
    tma::mbar_init(&s.bar[1], 1);
    if (GROUPS == 2 && grp == 0) tma::mbar_init(&s.go, 1);
    tma::fence_mbar_init();
  }
  __syncthreads();
  bool released = GROUPS == 1 || grp == 1;
  if (item >= total) {
    if (!released && tid == 0) tma::mbar_arrive(&sm[0].go);
    return;
  }
  if (GROUPS == 2 && grp == 1) tma::mbar_wait(&sm[0].go, 0, &args[0].sc->wait_error);

  auto issue = [&](int it, int k, float *dst, uint64_t *bar) {
    const HydroStepArgs &A = args[k];
    const int tile = it - (ENS ? pf[k] : 0);
    const int t1 = tile / A.nt0, t0 = tile - t1 * A.nt0;
    const CUtensorMap *tk = ENS ? table + (size_t)k * 4 : nullptr;
    const FieldRefs r{ENS ? tk : m0,
                      ENS ? tk + 1 : m1,
                      ENS ? tk + 2 : m2,
                      ENS ? tk + 3 : m3,
                      (const float *)A.rho,
                      (const float *)A.v0,
                      (const float *)A.v1,
                      (const float *)A.p};
    issue_box<NTH>(dst, box_inside(t0 * TX, t1 * TY, A.n0, A.n1), r, A.n0, A.n1, t0 * TX,
                   t1 * TY, bar, tid);
  };

  // sound speeds of the box cells into s.cq.c: items [i0, BH*BW/ (PAIR ? 2 : 1))
  // taken by threads t0.. with stride st
  auto sounds = [&](const float *Bx, const hf::Consts<float> &Kx, int first, int stride) {
    if (PAIR) {
      const hf::K<f2> k2 = hf::kconsts<f2>(Kx);
      for (int i = first; i < BH * BW / 2; i += stride) {
        const int j = i + BH * BW / 2;
        const f2 c = hf::sound(k2, hf::pack(Bx[i], Bx[j]),
                               hf::pack(Bx[3 * PLANE + i], Bx[3 * PLANE + j]));
        hf::unpack(c, s.cq.c[i], s.cq.c[j]);
      }
    } else {
      for (int i = first; i < BH * BW; i += stride)
        s.cq.c[i] = hf::sound(Kx, Bx[i], Bx[3 * PLANE + i]);
    }
  };
  // wait until the box of tile (X0, Y0) of an n0 x n1 grid has landed in
  // buffer bb (the caller synchronises the block afterwards)
  uint32_t parity = 0;  // bit k: parity of the next completed phase of bar[k]
  auto await_box = [&](int bb, int X0, int Y0, int n0, int n1, uint32_t *err) {
    if (box_inside(X0, Y0, n0, n1)) {
      tma::mbar_wait(&s.bar[bb], (parity >> bb) & 1u, err);
      parity ^= 1u << bb;
    } else {
      hk::cp_async_wait_all();
    }
  };
  auto tile_origin = [&](int it, int k, int &X0, int &Y0) {
    const HydroStepArgs &A = args[k];
    const int tile = it - (ENS ? pf[k] : 0);
    const int t1 = tile / A.nt0;
    X0 = (tile - t1 * A.nt0) * TX;
    Y0 = t1 * TY;
  };

  int lo = 0;  // instance of `item`
  if (ENS)
    while (lo < count - 1 && pf[lo + 1] <= item) ++lo;
  issue(item, lo, s.box[0], &s.bar[0]);
  if (ENS && warp == 0) copy_args(&s.args[0], &args[lo], lane);
  {
    int X0, Y0;
    tile_origin(item, lo, X0, Y0);
    await_box(0, X0, Y0, args[lo].n0, args[lo].n1, &args[lo].sc->wait_error);
    sync();
    sounds(s.box[0], hf::consts<float>(args[lo].gamma_f), tid, NTH);
  }
  sync();
  int b = 0;
  unsigned long long m = ~0ull;

  for (;;) {
    const HydroStepArgs &A = ENS ? s.args[b] : args[lo];
    const int n0 = A.n0, n1 = A.n1;
    const int tile = item - (ENS ? pf[lo] : 0);
    int X0, Y0;
    tile_origin(item, lo, X0, Y0);
    const float g = A.gamma_f;
    const hf::Consts<float> K = hf::consts<float>(g);
    const float dR0 = A.sc->dR0_f, dR1 = A.sc->dR1_f;
    const float dtG = hk::step_dt<float>(A);
    const float dtHalf = dtG / 2.0f;
    const float *B = s.box[b];

    // the next item's box goes into the other buffer while this one computes
    // (that buffer's last reader, the previous tile's stage 2, is behind the
    // last barrier)
    const int next = item + stride;
    int lo_n = lo;
    if (next < total) {
      if (ENS)
        while (lo_n < count - 1 && pf[lo_n + 1] <= next) ++lo_n;
      issue(next, lo_n, s.box[b ^ 1], &s.bar[b ^ 1]);
    }

    // stage-1 walls, order-1 reconstruction
    if (PAIR) {
      const hf::K<f2> k2 = hf::kconsts<f2>(K);
      for (int i = tid; i < kS1Half; i += NTH) {
        int axa, ca, wa, axb, cb, wb;
        s1_item(i, axa, ca, wa);
        const bool two = i + kS1Half < kS1Items;
        s1_item(two ? i + kS1Half : i, axb, cb, wb);
        const int da = axa == 0 ? 1 : BW, db = axb == 0 ? 1 : BW;
        const hf::NS<f2> L = pair_state(B, ca, axa, cb, axb);
        const hf::NS<f2> R = pair_state(B, ca + da, axa, cb + db, axb);
        const f2 cl = hf::pack(s.cq.c[ca], s.cq.c[cb]);
        const f2 cr = hf::pack(s.cq.c[ca + da], s.cq.c[cb + db]);
        Flux fa, fb;
        store_pair(hf::hllc_ns<f2>(k2, L, cl, R, cr), &fa, axa, &fb, axb);
        (axa == 0 ? s.fl.s1.x[wa] : s.fl.s1.y[wa]) = fa;
        if (two) (axb == 0 ? s.fl.s1.x[wb] : s.fl.s1.y[wb]) = fb;
      }
    } else {
      for (int i = tid; i < kS1Items; i += NTH) {
        int ax, c, w;
        s1_item(i, ax, c, w);
        if (ax == 0)
          s.fl.s1.x[w] =
              hf::hllc<0>(K, box_cell(B, c), s.cq.c[c], box_cell(B, c + 1), s.cq.c[c + 1]);
        else
          s.fl.s1.y[w] =
              hf::hllc<1>(K, box_cell(B, c), s.cq.c[c], box_cell(B, c + BW), s.cq.c[c + BW]);
      }
    }
    sync();

    // stage-1 cells (qy, qx) = box cell (qy+1, qx+2), advanced by dt/2
    {
      const float dtdx0 = dtHalf / dR0, dtdx1 = dtHalf / dR1;
      auto tape_cell = [&](int qy, int qx, const float *q, const Flux &l0, const Flux &r0,
                           const Flux &l1, const Flux &r1) {
        const int ty = qy - 2, tx = qx - 2;
        if (ty >= 0 && ty < TY && tx >= 0 && tx < TX) {
          const size_t gi = (size_t)(Y0 + ty) * n0 + (X0 + tx);
#pragma unroll
          for (int f = 0; f < 4; ++f) ((float *)tape->q[f])[gi] = q[f];
          hk::tape_diffs<float>(tape->d1, gi, l0, r0, l1, r1);
        }
      };
      if (PAIR) {
        const hf::K<f2> k2 = hf::kconsts<f2>(K);
        const f2 t0 = hf::splat<f2>(dtdx0), t1 = hf::splat<f2>(dtdx1);
        for (int i = tid; i < kQHalf; i += NTH) {
          int qya, qxa, qyb, qxb;
          q_item(i, qya, qxa);
          const bool two = i + kQHalf < kQItems;
          q_item(two ? i + kQHalf : i, qyb, qxb);
          const int ca = (qya + 1) * BW + qxa + 2, cb = (qyb + 1) * BW + qxb + 2;
          const Flux &l0a = s.fl.s1.x[qya * F1X + qxa], &r0a = s.fl.s1.x[qya * F1X + qxa + 1];
          const Flux &l1a = s.fl.s1.y[qya * F1Y + qxa], &r1a = s.fl.s1.y[(qya + 1) * F1Y + qxa];
          const Flux &l0b = s.fl.s1.x[qyb * F1X + qxb], &r0b = s.fl.s1.x[qyb * F1X + qxb + 1];
          const Flux &l1b = s.fl.s1.y[qyb * F1Y + qxb], &r1b = s.fl.s1.y[(qyb + 1) * F1Y + qxb];
          f2 q[4];
          hf::update_t<f2>(k2, hf::pack(B[ca], B[cb]), hf::pack(B[PLANE + ca], B[PLANE + cb]),
                           hf::pack(B[2 * PLANE + ca], B[2 * PLANE + cb]),
                           hf::pack(B[3 * PLANE + ca], B[3 * PLANE + cb]), t0, t1,
                           pack_flux(l0a, l0b), pack_flux(r0a, r0b), pack_flux(l1a, l1b),
                           pack_flux(r1a, r1b), q);
          float qa[4], qb[4];
#pragma unroll
          for (int f = 0; f < 4; ++f) hf::unpack(q[f], qa[f], qb[f]);
          if (TAPE) {
            tape_cell(qya, qxa, qa, l0a, r0a, l1a, r1a);
            if (two) tape_cell(qyb, qxb, qb, l0b, r0b, l1b, r1b);
          }
          s.cq.q[qya * QP + qxa] = make_float4(qa[0], qa[1], qa[2], qa[3]);
          if (two) s.cq.q[qyb * QP + qxb] = make_float4(qb[0], qb[1], qb[2], qb[3]);
        }
      } else {
        for (int i = tid; i < kQItems; i += NTH) {
          int qy, qx;
          q_item(i, qy, qx);
          const int c = (qy + 1) * BW + qx + 2;
          const Flux &l0 = s.fl.s1.x[qy * F1X + qx], &r0 = s.fl.s1.x[qy * F1X + qx + 1];
          const Flux &l1 = s.fl.s1.y[qy * F1Y + qx], &r1 = s.fl.s1.y[(qy + 1) * F1Y + qx];
          const Prim q = hf::update(K, box_cell(B, c), dtdx0, dtdx1, l0, r0, l1, r1);
          if (TAPE) {
            const float qv[4] = {q.rho, q.v0, q.v1, q.p};
            tape_cell(qy, qx, qv, l0, r0, l1, r1);
          }
          s.cq.q[qy * QP + qx] = make_float4(q.rho, q.v0, q.v1, q.p);
        }
      }
    }
    sync();
    if (!released) {  // group 0, first tile: let group 1 start
      if (tid == 0) tma::mbar_arrive(&sm[0].go);
      released = true;
    }

    // stage-2 walls, MUSCL-minmod of the stage-1 state: the x walls
    // 3t..3t+2 of row `lane` and the y walls 3t..3t+2 of column `lane`
    if (PAIR) {
      wall_run2(s.cq.q, (lane + 2) * QP + 3 * warp, 3 * warp * QP + lane + 2,
                &s.fl.s2.x[lane * F2X + 3 * warp], &s.fl.s2.y[3 * warp * F2Y + lane],
                hf::kconsts<f2>(K));
    } else if (warp < 11) {
      wall_run<0>(s.cq.q, (lane + 2) * QP + 3 * warp, 1, &s.fl.s2.x[lane * F2X + 3 * warp], 1, g,
                  K);
    } else {
      const int t = warp - 11;
      wall_run<1>(s.cq.q, 3 * t * QP + lane + 2, QP, &s.fl.s2.y[3 * t * F2Y + lane], F2Y, g, K);
    }
    // the next box must have landed before its sound speeds are formed
    if (next < total) {
      int Xn, Yn;
      tile_origin(next, lo_n, Xn, Yn);
      await_box(b ^ 1, Xn, Yn, args[lo_n].n0, args[lo_n].n1, &args[lo_n].sc->wait_error);
    }
    sync();

    // stage-2 cells (oy, ox) = box cell (oy+3, ox+4), advanced by dt and
    // written out, with the CFL minimum of the new state; the threads with
    // one stage-2 item form the next box's sound speeds (the stage-1 state
    // they overwrite was last read before the barrier above)
    {
      constexpr int P4 = PAIR ? TX * TY / 2 : TX * TY;  // stage-2 items
      constexpr int ONE = P4 - NTH;  // threads from here on take one item
      const float dtdx0 = dtG / dR0, dtdx1 = dtG / dR1;
      float *out[4] = {(float *)A.nrho, (float *)A.nv0, (float *)A.nv1, (float *)A.np};
      auto put = [&](int oy, int ox, const float *q, const float *cons, const Flux &l0,
                     const Flux &r0, const Flux &l1, const Flux &r1) {
        const size_t gi = (size_t)(Y0 + oy) * n0 + (X0 + ox);
        if (TAPE) {
          hk::tape_diffs<float>(tape->d2, gi, l0, r0, l1, r1);
#pragma unroll
          for (int k = 0; k < 4; ++k) ((float *)tape->u2[k])[gi] = cons[k];
        }
#pragma unroll
        for (int f = 0; f < 4; ++f) out[f][gi] = q[f];
        const float t = hs::timescale(g, dR0, dR1, q[0], q[1], q[2], q[3]);
        const unsigned long long bits = hk::ts_bits<float>(t);
        m = bits < m ? bits : m;
      };
      if (PAIR) {
        const hf::K<f2> k2 = hf::kconsts<f2>(K);
        const f2 t0 = hf::splat<f2>(dtdx0), t1 = hf::splat<f2>(dtdx1);
        for (int i = tid; i < P4; i += NTH) {
          const int oya = i >> 5, ox = i & 31, oyb = oya + TY / 2;
          const int ca = (oya + 3) * BW + ox + 4, cb = ca + (TY / 2) * BW;
          const Flux &l0a = s.fl.s2.x[oya * F2X + ox], &r0a = s.fl.s2.x[oya * F2X + ox + 1];
          const Flux &l1a = s.fl.s2.y[oya * F2Y + ox], &r1a = s.fl.s2.y[(oya + 1) * F2Y + ox];
          const Flux &l0b = s.fl.s2.x[oyb * F2X + ox], &r0b = s.fl.s2.x[oyb * F2X + ox + 1];
          const Flux &l1b = s.fl.s2.y[oyb * F2Y + ox], &r1b = s.fl.s2.y[(oyb + 1) * F2Y + ox];
          f2 q[4], cons[4];
          hf::update_t<f2>(k2, hf::pack(B[ca], B[cb]), hf::pack(B[PLANE + ca], B[PLANE + cb]),
                           hf::pack(B[2 * PLANE + ca], B[2 * PLANE + cb]),
                           hf::pack(B[3 * PLANE + ca], B[3 * PLANE + cb]), t0, t1,
                           pack_flux(l0a, l0b), pack_flux(r0a, r0b), pack_flux(l1a, l1b),
                           pack_flux(r1a, r1b), q, TAPE ? cons : nullptr);
          float qa[4], qb[4], ca4[4], cb4[4];
#pragma unroll
          for (int f = 0; f < 4; ++f) {
            hf::unpack(q[f], qa[f], qb[f]);
            if (TAPE) hf::unpack(cons[f], ca4[f], cb4[f]);
          }
          put(oya, ox, qa, ca4, l0a, r0a, l1a, r1a);
          put(oyb, ox, qb, cb4, l0b, r0b, l1b, r1b);
        }
      } else {
        for (int i = tid; i < P4; i += NTH) {
          const int oy = i >> 5, ox = i & 31;
          const int c = (oy + 3) * BW + ox + 4;
          const Flux &l0 = s.fl.s2.x[oy * F2X + ox], &r0 = s.fl.s2.x[oy * F2X + ox + 1];
          const Flux &l1 = s.fl.s2.y[oy * F2Y + ox], &r1 = s.fl.s2.y[(oy + 1) * F2Y + ox];
          float cons[4];
          const Prim q =
              hf::update(K, box_cell(B, c), dtdx0, dtdx1, l0, r0, l1, r1, TAPE ? cons : nullptr);
          const float qv[4] = {q.rho, q.v0, q.v1, q.p};
          put(oy, ox, qv, cons, l0, r0, l1, r1);
        }
      }
      if (next < total && tid >= ONE)
        sounds(s.box[b ^ 1], hf::consts<float>(args[lo_n].gamma_f), tid - ONE, NTH - ONE);
    }
    if (tile == 0 && tid == 0) {
      A.dt_hist[0] = (double)dtG;
      A.sc->dt_last = (double)dtG;
      A.sc->time = A.sc->time + (double)dtG;
    }
    // the next item's arguments into the other slot (its last reader, the
    // previous item, is behind the last barrier)
    if (ENS && next < total && warp == NTH / 32 - 1) copy_args(&s.args[b ^ 1], &args[lo_n], lane);
    // publish the CFL minimum when this CTA leaves the instance (the
    // reduction ends with a barrier); else one barrier before the next tile
    if (next >= total || lo_n != lo) {
      min_to(m, &A.sc->tsmin[1 - A.read_slot]);
      m = ~0ull;
    } else {
      sync();
    }
    if (next >= total) break;
    item = next;
    lo = lo_n;
    b ^= 1;
  }
}

template <bool TAPE>
__global__ void __launch_bounds__(NT, 2)
hydro_persist_kernel(HydroStepArgs a, const __grid_constant__ CUtensorMap m0,
                     const __grid_constant__ CUtensorMap m1,
                     const __grid_constant__ CUtensorMap m2,
                     const __grid_constant__ CUtensorMap m3, HydroTapeOut tape) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  persist_run<TAPE, false, false>(&a, nullptr, 1, nullptr, &m0, &m1, &m2, &m3,
                                  reinterpret_cast<Smem *>(smem_raw), &tape);
}

template <bool TAPE>
__global__ void __launch_bounds__(NT2, 2)
hydro_pair_kernel(HydroStepArgs a, const __grid_constant__ CUtensorMap m0,
                  const __grid_constant__ CUtensorMap m1, const __grid_constant__ CUtensorMap m2,
                  const __grid_constant__ CUtensorMap m3, HydroTapeOut tape) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  persist_run<TAPE, false, true>(&a, nullptr, 1, nullptr, &m0, &m1, &m2, &m3,
                                 reinterpret_cast<Smem *>(smem_raw), &tape);
}

// the paired form as one CTA per SM of two groups half a tile apart (two
// shared-memory blocks); 80 registers keep the 22 warps within the SM
// sub-partitions' register files
template <bool TAPE>
__global__ void __maxnreg__(80)
hydro_pair2_kernel(HydroStepArgs a, const __grid_constant__ CUtensorMap m0,
                   const __grid_constant__ CUtensorMap m1, const __grid_constant__ CUtensorMap m2,
                   const __grid_constant__ CUtensorMap m3, HydroTapeOut tape) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  persist_run<TAPE, false, true, 2>(&a, nullptr, 1, nullptr, &m0, &m1, &m2, &m3,
                                    reinterpret_cast<Smem *>(smem_raw), &tape);
}

// the paired ensemble step as one CTA per SM of two groups half an item apart
__global__ void __maxnreg__(80)
hydro_pair2_ensemble_kernel(const HydroStepArgs *__restrict__ args,
                            const int *__restrict__ prefix, int count,
                            const CUtensorMap *__restrict__ table) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  persist_run<false, true, true, 2>(args, prefix, count, table, nullptr, nullptr, nullptr, nullptr,
                                    reinterpret_cast<Smem *>(smem_raw), nullptr);
}

// table: 4 tensor maps per instance for the buffers `args` reads
template <bool PAIR>
__global__ void __launch_bounds__(PAIR ? NT2 : NT, 2)
hydro_persist_ensemble_kernel(const HydroStepArgs *__restrict__ args,
                              const int *__restrict__ prefix, int count,
                              const CUtensorMap *__restrict__ table) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  persist_run<false, true, PAIR>(args, prefix, count, table, nullptr, nullptr, nullptr, nullptr,
                                 reinterpret_cast<Smem *>(smem_raw), nullptr);
}

}  // namespace hp
}  // namespace om

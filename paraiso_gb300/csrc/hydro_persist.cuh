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
//    of a row (or column) are 11 runs, so the 704 walls-runs of a tile are
//    exactly one per thread of the 704-thread CTA.
//  * The tile's CFL minimum is folded in registers over all the tiles of a
//    CTA (of one instance) and published once.
// Every value is formed by the same expressions as the production tile
// kernel of hydro_kernels.cuh, so the two give the same bits.
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
  unsigned long long red[32];
};

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
__device__ __forceinline__ void issue_box(float *dst, bool inside, const CUtensorMap *const *maps,
                                          const float *const *f, int n0, int n1, int X0, int Y0,
                                          uint64_t *bar) {
  if (inside) {
    if (threadIdx.x == 0) {
      tma::fence_proxy_async();
      tma::mbar_arrive_expect_tx(bar, kBoxBytes);
#pragma unroll
      for (int k = 0; k < 4; ++k) tma::load_2d(dst + k * PLANE, maps[k], X0 - 4, Y0 - 3, bar);
    }
  } else {
    for (int i = threadIdx.x; i < BH * 10; i += NT) {
      const int py = i / 10, j = i - py * 10;
      const int gy = hk::wrap_near(Y0 - 3 + py, n1), gx = hk::wrap_near(X0 - 4 + 4 * j, n0);
      const size_t gi = (size_t)gy * n0 + gx;
      float *d = dst + py * BW + 4 * j;
#pragma unroll
      for (int k = 0; k < 4; ++k) cp_async16(d + k * PLANE, f[k] + gi);
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
// q[base + j st .. base + (j+3) st] (hs::muscl); its flux goes to
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
      (&L.rho)[f] = b + hs::absmaller(b - a, c - b) / 2.0f;
    }
  }
  float cl = hs::sound(g, L.rho, L.p);
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const Prim x1 = rec(q[base + (j + 1) * st]), x2 = rec(q[base + (j + 2) * st]),
               x3 = rec(q[base + (j + 3) * st]);
    Prim R, Ln;
#pragma unroll
    for (int f = 0; f < 4; ++f) {
      const float b = (&x1.rho)[f], c = (&x2.rho)[f], d = (&x3.rho)[f];
      const float s = hs::absmaller(c - b, d - c);
      (&R.rho)[f] = c - s / 2.0f;
      (&Ln.rho)[f] = c + s / 2.0f;
    }
    const float cr = hs::sound(g, R.rho, R.p);
    out[j * ost] = hf::hllc<AX>(K, L, cl, R, cr);
    if (j < 2) {
      L = Ln;
      cl = hs::sound(g, L.rho, L.p);
    }
  }
}

// The tiles of one grid (ENS false: args[0], maps m[0..3]) or of an
// ensemble (ENS true: instance k has args[k], maps table[(k * 4) + field]
// and items pf[k] .. pf[k+1]-1).  TAPE: the taped step (single grid).
template <bool TAPE, bool ENS>
__device__ __forceinline__ void persist_run(const HydroStepArgs *__restrict__ args,
                                            const int *__restrict__ pf, int count,
                                            const CUtensorMap *table, const CUtensorMap *m0,
                                            const CUtensorMap *m1, const CUtensorMap *m2,
                                            const CUtensorMap *m3, Smem &s,
                                            const HydroTapeOut *tape) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int total =
      ENS ? pf[count] : args[0].nt0 * ((args[0].n1 + TY - 1) / TY);
  int item = blockIdx.x;
  if (item >= total) return;
  if (tid == 0) {
    tma::mbar_init(&s.bar[0], 1);
    tma::mbar_init(&s.bar[1], 1);
    tma::fence_mbar_init();
  }
  __syncthreads();

  auto instance_maps = [&](int k, const CUtensorMap **mp) {
    if (ENS) {
#pragma unroll
      for (int f = 0; f < 4; ++f) mp[f] = table + (size_t)k * 4 + f;
    } else {
      mp[0] = m0; mp[1] = m1; mp[2] = m2; mp[3] = m3;
    }
  };
  auto issue = [&](int it, int k, float *dst, uint64_t *bar) {
    const HydroStepArgs &A = args[k];
    const int tile = it - (ENS ? pf[k] : 0);
    const int t1 = tile / A.nt0, t0 = tile - t1 * A.nt0;
    const float *f[4] = {(const float *)A.rho, (const float *)A.v0, (const float *)A.v1,
                         (const float *)A.p};
    const CUtensorMap *mp[4];
    instance_maps(k, mp);
    issue_box(dst, box_inside(t0 * TX, t1 * TY, A.n0, A.n1), mp, f, A.n0, A.n1, t0 * TX, t1 * TY,
              bar);
  };

  int lo = 0;  // instance of `item`
  if (ENS)
    while (lo < count - 1 && pf[lo + 1] <= item) ++lo;
  issue(item, lo, s.box[0], &s.bar[0]);
  int b = 0;
  uint32_t parity = 0;  // bit k: parity of the next completed phase of bar[k]
  unsigned long long m = ~0ull;

  for (;;) {
    const HydroStepArgs &A = args[lo];
    const int n0 = A.n0, n1 = A.n1;
    const int tile = item - (ENS ? pf[lo] : 0);
    const int t1 = tile / A.nt0, t0 = tile - t1 * A.nt0;
    const int X0 = t0 * TX, Y0 = t1 * TY;
    const float g = A.gamma_f;
    const hf::Consts<float> K = hf::consts<float>(g);
    const float dR0 = A.sc->dR0_f, dR1 = A.sc->dR1_f;
    const float dtG = hk::step_dt<float>(A);
    const float dtHalf = dtG / 2.0f;

    // this tile's box has landed
    if (box_inside(X0, Y0, n0, n1)) {
      tma::mbar_wait(&s.bar[b], (parity >> b) & 1u, &A.sc->wait_error);
      parity ^= 1u << b;
    } else {
      hk::cp_async_wait_all();
    }
    __syncthreads();
    const float *B = s.box[b];

    // sound speeds of the box cells
    for (int i = tid; i < BH * BW; i += NT) s.cq.c[i] = hs::sound(g, B[i], B[3 * PLANE + i]);
    __syncthreads();

    // the next item's box goes into the other buffer while this one computes
    const int next = item + gridDim.x;
    int lo_n = lo;
    if (next < total) {
      if (ENS)
        while (lo_n < count - 1 && pf[lo_n + 1] <= next) ++lo_n;
      issue(next, lo_n, s.box[b ^ 1], &s.bar[b ^ 1]);
    }

    // stage-1 walls, order-1 reconstruction (x wall fx of row fy between box
    // cells (fy+1, fx+1) and (fy+1, fx+2); y wall fx of row fy between
    // (fy, fx+2) and (fy+1, fx+2))
    for (int i = tid; i < kS1Items; i += NT) {
      int ax, fy, fx;
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
      if (ax == 0) {
        const int c = (fy + 1) * BW + fx + 1;
        s.fl.s1.x[fy * F1X + fx] =
            hf::hllc<0>(K, box_cell(B, c), s.cq.c[c], box_cell(B, c + 1), s.cq.c[c + 1]);
      } else {
        const int c = fy * BW + fx + 2;
        s.fl.s1.y[fy * F1Y + fx] =
            hf::hllc<1>(K, box_cell(B, c), s.cq.c[c], box_cell(B, c + BW), s.cq.c[c + BW]);
      }
    }
    __syncthreads();

    // stage-1 cells (qy, qx) = box cell (qy+1, qx+2), advanced by dt/2
    {
      const float dtdx0 = dtHalf / dR0, dtdx1 = dtHalf / dR1;
      for (int i = tid; i < kQItems; i += NT) {
        int qy, qx;
        if (i < kQMain) {
          qy = i >> 5; qx = i & 31;
        } else {
          const int j = i - kQMain;
          qy = j >> 2; qx = 32 + (j & 3);
        }
        const int c = (qy + 1) * BW + qx + 2;
        const Flux &l0 = s.fl.s1.x[qy * F1X + qx], &r0 = s.fl.s1.x[qy * F1X + qx + 1];
        const Flux &l1 = s.fl.s1.y[qy * F1Y + qx], &r1 = s.fl.s1.y[(qy + 1) * F1Y + qx];
        const Prim q = hf::update(K, box_cell(B, c), dtdx0, dtdx1, l0, r0, l1, r1);
        if (TAPE) {
          const int ty = qy - 2, tx = qx - 2;
          if (ty >= 0 && ty < TY && tx >= 0 && tx < TX) {
            const size_t gi = (size_t)(Y0 + ty) * n0 + (X0 + tx);
            ((float *)tape->q[0])[gi] = q.rho;
            ((float *)tape->q[1])[gi] = q.v0;
            ((float *)tape->q[2])[gi] = q.v1;
            ((float *)tape->q[3])[gi] = q.p;
            hk::tape_diffs<float>(tape->d1, gi, l0, r0, l1, r1);
          }
        }
        s.cq.q[qy * QP + qx] = make_float4(q.rho, q.v0, q.v1, q.p);
      }
    }
    __syncthreads();

    // stage-2 walls, MUSCL-minmod of the stage-1 state: warps 0-10 take
    // the x walls 3w..3w+2 of row `lane`, warps 11-21 the y walls
    // 3t..3t+2 of column `lane`
    if (warp < 11) {
      wall_run<0>(s.cq.q, (lane + 2) * QP + 3 * warp, 1, &s.fl.s2.x[lane * F2X + 3 * warp], 1, g,
                  K);
    } else {
      const int t = warp - 11;
      wall_run<1>(s.cq.q, 3 * t * QP + lane + 2, QP, &s.fl.s2.y[3 * t * F2Y + lane], F2Y, g, K);
    }
    __syncthreads();

    // stage-2 cells (oy, ox) = box cell (oy+3, ox+4), advanced by dt and
    // written out, with the CFL minimum of the new state
    {
      const float dtdx0 = dtG / dR0, dtdx1 = dtG / dR1;
      float *orho = (float *)A.nrho, *ovx = (float *)A.nv0, *ovy = (float *)A.nv1,
            *opr = (float *)A.np;
      for (int i = tid; i < TX * TY; i += NT) {
        const int oy = i >> 5, ox = i & 31;
        const int c = (oy + 3) * BW + ox + 4;
        const Flux &l0 = s.fl.s2.x[oy * F2X + ox], &r0 = s.fl.s2.x[oy * F2X + ox + 1];
        const Flux &l1 = s.fl.s2.y[oy * F2Y + ox], &r1 = s.fl.s2.y[(oy + 1) * F2Y + ox];
        float cons[4];
        const Prim q =
            hf::update(K, box_cell(B, c), dtdx0, dtdx1, l0, r0, l1, r1, TAPE ? cons : nullptr);
        const size_t gi = (size_t)(Y0 + oy) * n0 + (X0 + ox);
        if (TAPE) {
          hk::tape_diffs<float>(tape->d2, gi, l0, r0, l1, r1);
#pragma unroll
          for (int k = 0; k < 4; ++k) ((float *)tape->u2[k])[gi] = cons[k];
        }
        orho[gi] = q.rho;
        ovx[gi] = q.v0;
        ovy[gi] = q.v1;
        opr[gi] = q.p;
        const float t = hs::timescale(g, dR0, dR1, q.rho, q.v0, q.v1, q.p);
        const unsigned long long bits = hk::ts_bits<float>(t);
        m = bits < m ? bits : m;
      }
    }
    if (tile == 0 && tid == 0) {
      A.dt_hist[0] = (double)dtG;
      A.sc->dt_last = (double)dtG;
      A.sc->time = A.sc->time + (double)dtG;
    }
    // publish the CFL minimum when this CTA leaves the instance
    if (next >= total || lo_n != lo) {
      hk::block_min_to(m, &A.sc->tsmin[1 - A.read_slot], s.red);
      m = ~0ull;
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
  persist_run<TAPE, false>(&a, nullptr, 1, nullptr, &m0, &m1, &m2, &m3,
                           *reinterpret_cast<Smem *>(smem_raw), &tape);
}

// table: 4 tensor maps per instance for the buffers `args` reads
__global__ void __launch_bounds__(NT, 2)
hydro_persist_ensemble_kernel(const HydroStepArgs *__restrict__ args,
                              const int *__restrict__ prefix, int count,
                              const CUtensorMap *__restrict__ table) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  persist_run<false, true>(args, prefix, count, table, nullptr, nullptr, nullptr, nullptr,
                           *reinterpret_cast<Smem *>(smem_raw), nullptr);
}

}  // namespace hp
}  // namespace om

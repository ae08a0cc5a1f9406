// life.cu -- Conway's Life Orthotope Machine on GB300.
//
// Reference: examples/Life/Generator.hs:67-115 (init, proceed), the
// generated loop examples-old/Life-exampled/dist/Life.cpp:114-183 and the
// CPU/GPU reduce library (Language/Paraiso/Generator/PlanTrans.hs:712-720).
//
//   proceed:  num   = sum of the 8 shifted copies of cell
//             alive = (cell==0 && num==3) || (cell==1 && num>=2 && num<=3)
//             cell' = alive ? 1 : 0
//             population = reduce Sum cell'      generation = generation + 1
//
// Three device paths give bit-identical results:
//  * life_general_kernel: one int32 cell per thread with the reference's
//    integer arithmetic; any size, cyclic or open boundary, any cell values.
//  * life_smallgrid_kernel: whole grid bit-packed in shared memory (one CTA),
//    all generations of a run in one launch.  Cyclic, width % 32 == 0.
//  * life_tb_kernel: bit-packed tiles with a 1-word / k-row halo, k
//    generations per launch (temporal blocking).  Cyclic, width % 32 == 0.
// The packed paths require every cell in {0,1}; then num is in [0,8] and
// the rule equals the bit-sliced adder below, so outputs are identical.
// After any external write the first generation runs on the general path,
// whose outputs are always 0/1.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <string>

#include "om_internal.cuh"
#include "tma.cuh"

namespace om {

struct LifeScalars {  // device/host scalar block
  int32_t population;
  int32_t generation;
  uint32_t wait_error;  // raised by a kernel whose bounded wait ran out
};

struct LifeState {
  bool binary = true;           // every cell is known to be 0 or 1
  uint32_t *d_pop = nullptr;    // populations of the last run, per generation
  uint32_t *d_flag = nullptr;   // raised by the cell-value check
  int pop_cap = 0;
  int last_n = 0;
  int depth = 0, tile_w = 0, tile_h = 0;  // tuned or configured
  // tensor maps of the two cell buffers (cells x words x rows) for the TMA
  // kernels, keyed by buffer address, and their one-word maps (32 cells x 1
  // word x 1 row, no swizzle) for the halo word that wraps around;
  // tmap_ok[i] false when encoding failed
  CUtensorMap tmap[2], tpatch[2];
  const void *tmap_ptr[2] = {nullptr, nullptr};
  bool tmap_ok[2] = {false, false};
};

// Index of the cached maps of cell buffer `cells` (n0 x n1 int32, n0 a
// multiple of 32), -1 when the driver does not encode them: dimensions 32
// cells x n0/32 words x n1 rows, boxes of one row of 32 words with 128-byte
// swizzle (st->tmap[i]) and of one word (st->tpatch[i]).
static int life_tmap(LifeState *st, const void *cells, int n0, int n1) {
  for (int i = 0; i < 2; ++i)
    if (st->tmap_ptr[i] == cells) return st->tmap_ok[i] ? i : -1;
  const int i = st->tmap_ptr[0] == nullptr ? 0 : (st->tmap_ptr[1] == nullptr ? 1 : 0);
  const uint64_t dims[3] = {32, (uint64_t)(n0 / 32), (uint64_t)n1};
  const uint64_t strides[2] = {128, (uint64_t)n0 * 4};
  const uint32_t box[3] = {32, 32, 1}, box1[3] = {32, 1, 1};
  st->tmap_ptr[i] = cells;
  st->tmap_ok[i] = tma::encode_tiled(&st->tmap[i], CU_TENSOR_MAP_DATA_TYPE_INT32, 3,
                                     const_cast<void *>(cells), dims, strides, box,
                                     CU_TENSOR_MAP_SWIZZLE_128B) &&
                   tma::encode_tiled(&st->tpatch[i], CU_TENSOR_MAP_DATA_TYPE_INT32, 3,
                                     const_cast<void *>(cells), dims, strides, box1,
                                     CU_TENSOR_MAP_SWIZZLE_NONE);
  return st->tmap_ok[i] ? i : -1;
}

static LifeState *life_state(Handle *h) { return (LifeState *)h->impl; }

cudaError_t life_check_cells_into(const int32_t *cells, size_t n, uint32_t *flag,
                                  cudaStream_t s);

// ---------------------------------------------------------------------------
// device code
// ---------------------------------------------------------------------------

// Next state of 32 cells (one word, bit i = cell 32w+i) from the words of
// the row above (a), the row itself (b) and the row below (c), each with its
// left (L) and right (R) neighbour word.
__device__ __forceinline__ uint32_t life_word(uint32_t aL, uint32_t a, uint32_t aR,
                                              uint32_t bL, uint32_t b, uint32_t bR,
                                              uint32_t cL, uint32_t c, uint32_t cR) {
  const uint32_t aW = __funnelshift_l(aL, a, 1), aE = __funnelshift_r(a, aR, 1);
  const uint32_t bW = __funnelshift_l(bL, b, 1), bE = __funnelshift_r(b, bR, 1);
  const uint32_t cW = __funnelshift_l(cL, c, 1), cE = __funnelshift_r(c, cR, 1);
  // column sums as 2-bit numbers: row a (3 cells), row b (2 cells), row c
  const uint32_t a1 = aW ^ a ^ aE, a2 = (aW & a) | (aE & (aW ^ a));
  const uint32_t c1 = cW ^ c ^ cE, c2 = (cW & c) | (cE & (cW ^ c));
  const uint32_t b1 = bW ^ bE, b2 = bW & bE;
  // num = s0 + 2*(a2 + b2 + c2 + k0)
  const uint32_t s0 = a1 ^ b1 ^ c1;
  const uint32_t k0 = (a1 & b1) | (c1 & (a1 ^ b1));
  // alive' = (num == 3) | (b & num == 2) = exactly-one(a2,b2,c2,k0) & (s0 | b)
  const uint32_t one = (a2 ^ b2 ^ c2 ^ k0) & ~(a2 & b2) & ~(c2 & k0);
  return one & (s0 | b);
}

// One generation on int32 cells, the reference's arithmetic.  Grid covers
// the memory array; open-boundary margins of `next` are written 0 (the
// generated manifest is never written there).
template <bool CYCLIC>
__global__ void __launch_bounds__(256)
life_general_kernel(const int32_t *__restrict__ cur, int32_t *__restrict__ next,
                    int ms0, int ms1, int lm, int tiles_x,
                    uint32_t *__restrict__ pop) {
  const int bx = (int)(blockIdx.x % (unsigned)tiles_x);
  const int by = (int)(blockIdx.x / (unsigned)tiles_x);
  const int x = bx * 32 + threadIdx.x;
  const int y = by * 8 + threadIdx.y;
  uint32_t v = 0;
  if (x < ms0 && y < ms1) {
    const bool interior =
        CYCLIC || (x >= lm && x < ms0 - lm && y >= lm && y < ms1 - lm);
    if (interior) {
      int xm, xp, ym, yp;
      if (CYCLIC) {
        xm = x == 0 ? ms0 - 1 : x - 1;
        xp = x == ms0 - 1 ? 0 : x + 1;
        ym = y == 0 ? ms1 - 1 : y - 1;
        yp = y == ms1 - 1 ? 0 : y + 1;
      } else {
        xm = x - 1; xp = x + 1; ym = y - 1; yp = y + 1;
      }
      const int32_t *rm = cur + (size_t)ym * ms0;
      const int32_t *r0 = cur + (size_t)y * ms0;
      const int32_t *rp = cur + (size_t)yp * ms0;
      // wraparound integer sum, as the generated int arithmetic
      const uint32_t num = (uint32_t)rp[xp] + (uint32_t)rp[x] + (uint32_t)rp[xm] +
                           (uint32_t)r0[xp] + (uint32_t)r0[xm] + (uint32_t)rm[xp] +
                           (uint32_t)rm[x] + (uint32_t)rm[xm];
      const int32_t n = (int32_t)num;
      const int32_t c = r0[x];
      v = ((c == 0 && n == 3) || (c == 1 && n >= 2 && n <= 3)) ? 1u : 0u;
    }
    next[(size_t)y * ms0 + x] = (int32_t)v;
  }
  __shared__ uint32_t ws[8];
  const uint32_t s = __reduce_add_sync(0xffffffffu, v);
  const int warp = threadIdx.y;
  if (threadIdx.x == 0) ws[warp] = s;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = threadIdx.x < 8 ? ws[threadIdx.x] : 0u;
    t = __reduce_add_sync(0xffffffffu, t);
    if (threadIdx.x == 0 && t) atomicAdd(pop, t);
  }
}

// Load an nr x nc block of packed words into shared memory (row stride nc):
// block row r is global row wrap(row0 + r), block column c is global word
// wrap(col0 + c).  One warp per row at a time; each word is 32 coalesced
// int32 loads folded by a ballot, 8 words in flight per warp.  Row and
// word indices advance incrementally (no division per word).
__device__ __forceinline__ void pack_rows(const int32_t *__restrict__ cur, int n0, int n1,
                                          int wd, int row0, int col0, int nc, int nr,
                                          uint32_t *dst, int warp, int nwarps, int lane) {
  int gx0 = col0 % wd;
  if (gx0 < 0) gx0 += wd;
  const bool narrow = nc > wd;  // tiny grids: a tile row wraps more than once
  for (int r = warp; r < nr; r += nwarps) {
    int gy = (row0 + r) % n1;
    if (gy < 0) gy += n1;
    const int32_t *row = cur + (size_t)gy * n0 + lane;
    uint32_t *out = dst + r * nc;
    for (int c0 = 0; c0 < nc; c0 += 8) {
      int32_t v[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int c = c0 + j;
        v[j] = 0;
        if (c < nc) {
          int gx = gx0 + c;
          if (narrow) gx %= wd;
          else if (gx >= wd) gx -= wd;
          v[j] = __ldg(row + (size_t)gx * 32);
        }
      }
      uint32_t mine = 0;
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const uint32_t w = __ballot_sync(0xffffffffu, v[j] != 0);
        if (lane == j) mine = w;
      }
      if (lane < 8 && c0 + lane < nc) out[c0 + lane] = mine;
    }
  }
}

// Bit t of an 8-bit value moved to bit 4t.
__device__ __forceinline__ uint32_t spread4(uint32_t x) {
  x = (x | (x << 12)) & 0x000F000Fu;
  x = (x | (x << 6)) & 0x03030303u;
  x = (x | (x << 3)) & 0x11111111u;
  return x;
}

// pack_rows with 128-bit cell loads: lane L reads cells 4(L%8)..4(L%8)+3 of
// word L/8 of a 4-word group, so one warp instruction moves 512 bytes.
// Ballot j holds cell 4t+j of word m at bit 8m+t; word m is the four bytes
// m of the ballots interleaved.  G groups (4G words, G x 512 bytes) in
// flight per warp.
template <int G>
__device__ __forceinline__ void pack_rows_vec(const int32_t *__restrict__ cur, int n0, int n1,
                                              int wd, int row0, int col0, int nc, int nr,
                                              uint32_t *dst, int warp, int nwarps, int lane) {
  int gx0 = col0 % wd;
  if (gx0 < 0) gx0 += wd;
  const bool narrow = nc > wd;
  const int sub = lane >> 3, quad = (lane & 7) * 4;
  for (int r = warp; r < nr; r += nwarps) {
    int gy = (row0 + r) % n1;
    if (gy < 0) gy += n1;
    const int32_t *row = cur + (size_t)gy * n0 + quad;
    uint32_t *out = dst + r * nc;
    for (int c0 = 0; c0 < nc; c0 += 4 * G) {
      int4 v[G];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const int cw = c0 + 4 * g + sub;
        v[g] = make_int4(0, 0, 0, 0);
        if (cw < nc) {
          int gx = gx0 + cw;
          if (narrow) gx %= wd;
          else if (gx >= wd) gx -= wd;
          v[g] = __ldg(reinterpret_cast<const int4 *>(row + (size_t)gx * 32));
        }
      }
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const uint32_t b0 = __ballot_sync(0xffffffffu, v[g].x != 0);
        const uint32_t b1 = __ballot_sync(0xffffffffu, v[g].y != 0);
        const uint32_t b2 = __ballot_sync(0xffffffffu, v[g].z != 0);
        const uint32_t b3 = __ballot_sync(0xffffffffu, v[g].w != 0);
        const int cw = c0 + 4 * g + lane;
        if (lane < 4 && cw < nc) {
          const int sh = 8 * lane;
          out[cw] = spread4((b0 >> sh) & 0xFFu) | (spread4((b1 >> sh) & 0xFFu) << 1) |
                    (spread4((b2 >> sh) & 0xFFu) << 2) | (spread4((b3 >> sh) & 0xFFu) << 3);
        }
      }
    }
  }
}

// pack_rows_vec for rows of exactly 32 words (the register kernel), for
// cells that are all 0 or 1: lane L loads cells 4t .. 4t+3 (t = L % 8) of
// word 4g + L / 8 of group g, forms their nibble shifted to bit 4t with
// multiply-adds, and the eight lanes of a word add their nibbles (disjoint
// bits) in three butterfly steps.  Lane 8s of each word's eight stores it.
__device__ __forceinline__ void pack_rows32(const int32_t *__restrict__ cur, int n0, int n1,
                                            int wd, int row0, int col0, int nr, uint32_t *dst,
                                            int warp, int nwarps, int lane) {
  int gx0 = col0 % wd;
  if (gx0 < 0) gx0 += wd;
  const bool narrow = 32 > wd;
  const int sub = lane >> 3, t = lane & 7, quad = t * 4;
  const uint32_t m1 = 1u << quad, m2 = m1 << 1, m4 = m1 << 2, m8 = m1 << 3;
  for (int r = warp; r < nr; r += nwarps) {
    int gy = (row0 + r) % n1;
    if (gy < 0) gy += n1;
    const int32_t *row = cur + (size_t)gy * n0 + quad;
    int4 v[8];
#pragma unroll
    for (int g = 0; g < 8; ++g) {
      int gx = gx0 + 4 * g + sub;
      if (narrow) gx %= wd;
      else if (gx >= wd) gx -= wd;
      v[g] = __ldg(reinterpret_cast<const int4 *>(row + (size_t)gx * 32));
    }
#pragma unroll
    for (int g = 0; g < 8; ++g) {
      uint32_t w = (uint32_t)v[g].x * m1 + (uint32_t)v[g].y * m2 + (uint32_t)v[g].z * m4 +
                   (uint32_t)v[g].w * m8;
      w += __shfl_xor_sync(0xffffffffu, w, 1);
      w += __shfl_xor_sync(0xffffffffu, w, 2);
      w += __shfl_xor_sync(0xffffffffu, w, 4);
      if (t == 0) dst[r * 32 + 4 * g + sub] = w;
    }
  }
}

// pack_rows32 with each lane's cells staged in shared memory by
// asynchronous 16-byte copies, two rows in flight per warp: the loads of the
// next row are under way while this row's nibbles are summed, and no
// registers are held by loads in flight.  A lane reads back only the cells it
// copied itself, so the warp needs no barrier.  `stage` is 2 x 256 int4 of
// this warp.
__device__ __forceinline__ void pack_rows32_async(const int32_t *__restrict__ cur, int n0, int n1,
                                                  int wd, int row0, int col0, int nr,
                                                  uint32_t *dst, int warp, int nwarps, int lane,
                                                  int4 *stage) {
  int gx0 = col0 % wd;
  if (gx0 < 0) gx0 += wd;
  const bool narrow = 32 > wd;
  const int sub = lane >> 3, t = lane & 7, quad = t * 4;
  const uint32_t m1 = 1u << quad, m2 = m1 << 1, m4 = m1 << 2, m8 = m1 << 3;
  auto issue = [&](int r, int4 *into) {
    int gy = (row0 + r) % n1;
    if (gy < 0) gy += n1;
    const int32_t *row = cur + (size_t)gy * n0 + quad;
#pragma unroll
    for (int g = 0; g < 8; ++g) {
      int gx = gx0 + 4 * g + sub;
      if (narrow) gx %= wd;
      else if (gx >= wd) gx -= wd;
      const unsigned d = (unsigned)__cvta_generic_to_shared(into + g * 32 + lane);
      asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d),
                   "l"(row + (size_t)gx * 32)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  int i = 0;
  if (warp < nr) issue(warp, stage);
  for (int r = warp; r < nr; r += nwarps, ++i) {
    int4 *cur_stage = stage + (i & 1) * 256;
    if (r + nwarps < nr) {
      issue(r + nwarps, stage + ((i + 1) & 1) * 256);
      asm volatile("cp.async.wait_group 1;\n" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    }
#pragma unroll
    for (int g = 0; g < 8; ++g) {
      const int4 v = cur_stage[g * 32 + lane];
      uint32_t w = (uint32_t)v.x * m1 + (uint32_t)v.y * m2 + (uint32_t)v.z * m4 +
                   (uint32_t)v.w * m8;
      w += __shfl_xor_sync(0xffffffffu, w, 1);
      w += __shfl_xor_sync(0xffffffffu, w, 2);
      w += __shfl_xor_sync(0xffffffffu, w, 4);
      if (t == 0) dst[r * 32 + 4 * g + sub] = w;
    }
  }
}

// Whole grid in shared memory: all `gens` generations in one launch.
__global__ void __launch_bounds__(512)
life_smallgrid_kernel(const int32_t *__restrict__ cur, int32_t *__restrict__ next,
                      int n0, int n1, int gens, uint32_t *__restrict__ pop) {
  extern __shared__ uint32_t sm[];
  __shared__ uint32_t spop[3];
  const int wd = n0 >> 5;
  const int nw = wd * n1;
  uint32_t *A = sm, *B = sm + nw;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nthreads = blockDim.x, nwarps = nthreads >> 5;
  pack_rows(cur, n0, n1, wd, 0, 0, wd, n1, A, warp, nwarps, lane);
  if (tid < 3) spop[tid] = 0;
  __syncthreads();
  for (int g = 0; g < gens; ++g) {
    uint32_t cnt = 0;
    for (int i = tid; i < nw; i += nthreads) {
      const int y = i / wd, x = i - y * wd;
      const int ym = (y == 0 ? n1 - 1 : y - 1) * wd, y0 = y * wd,
                yp = (y == n1 - 1 ? 0 : y + 1) * wd;
      const int xm = x == 0 ? wd - 1 : x - 1, xp = x == wd - 1 ? 0 : x + 1;
      const uint32_t r = life_word(A[ym + xm], A[ym + x], A[ym + xp],
                                   A[y0 + xm], A[y0 + x], A[y0 + xp],
                                   A[yp + xm], A[yp + x], A[yp + xp]);
      B[i] = r;
      cnt += __popc(r);
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if (lane == 0 && cnt) atomicAdd(&spop[g % 3], cnt);
    __syncthreads();
    if (tid == 0) {
      pop[g] = spop[g % 3];
      spop[(g + 2) % 3] = 0;
    }
    uint32_t *t = A; A = B; B = t;
  }
  // unpack: lane i of the warp writes bit i of the word
  for (int i = warp; i < nw; i += nwarps) {
    const int y = i / wd, x = i - y * wd;
    const uint32_t w = A[i];
    next[(size_t)y * n0 + (size_t)x * 32 + lane] = (int32_t)((w >> lane) & 1u);
  }
}

struct TbParams {
  int n0, n1, wd;   // grid in cells, width in words
  int tw, th, kk;   // tile width (words), height (rows), generations
  int nt0, nt1;     // tiles per axis
};

// Temporal blocking: each CTA owns a tw x th tile (words x rows), loads it
// with a halo of 1 word and kk rows, advances kk generations in shared
// memory and writes back its owned cells.  After g generations the halo's
// stale front has moved g cells / rows inward; kk <= 32 keeps it inside the
// halo word, and kk rows of vertical halo keep it off the owned rows.
template <bool VEC>
__global__ void __launch_bounds__(256)
life_tb_kernel(const int32_t *__restrict__ cur, int32_t *__restrict__ next,
               TbParams p, uint32_t *__restrict__ pop) {
  extern __shared__ uint32_t sm[];
  __shared__ uint32_t spop[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nthreads = blockDim.x, nwarps = nthreads >> 5;
  const int t = blockIdx.x;
  const int t0 = t % p.nt0, t1 = t / p.nt0;
  const int col0 = t0 * p.tw, row0 = t1 * p.th;
  const int tw_own = min(p.tw, p.wd - col0), th_own = min(p.th, p.n1 - row0);
  const int kk = p.kk;
  const int NC = tw_own + 2, NR = th_own + 2 * kk;
  const int stride = (p.tw + 2) * (p.th + 2 * kk);
  uint32_t *A = sm, *B = sm + stride;
  if (tid < 32) spop[tid] = 0;
  if (VEC)
    pack_rows_vec<4>(cur, p.n0, p.n1, p.wd, row0 - kk, col0 - 1, NC, NR, A, warp, nwarps, lane);
  else
    pack_rows(cur, p.n0, p.n1, p.wd, row0 - kk, col0 - 1, NC, NR, A, warp, nwarps, lane);
  __syncthreads();
  const int NG = max(1, nthreads / NC);
  for (int g = 1; g <= kk; ++g) {
    const int nrows = NR - 2 * g;
    const int chunk = (nrows + NG - 1) / NG;
    uint32_t cnt = 0;
    for (int ci = tid; ci < NC * NG; ci += nthreads) {
      const int c = ci % NC, grp = ci / NC;
      const int rs = g + grp * chunk, re = min(rs + chunk, NR - g);
      if (rs >= re) continue;
      const bool hasL = c > 0, hasR = c < NC - 1;
      const uint32_t *col = A + c;
      uint32_t aL = hasL ? col[(rs - 1) * NC - 1] : 0u, a = col[(rs - 1) * NC],
               aR = hasR ? col[(rs - 1) * NC + 1] : 0u;
      uint32_t bL = hasL ? col[rs * NC - 1] : 0u, b = col[rs * NC],
               bR = hasR ? col[rs * NC + 1] : 0u;
      const bool own_c = c >= 1 && c <= tw_own;
      for (int r = rs; r < re; ++r) {
        const uint32_t cL = hasL ? col[(r + 1) * NC - 1] : 0u, cc = col[(r + 1) * NC],
                       cR = hasR ? col[(r + 1) * NC + 1] : 0u;
        const uint32_t w = life_word(aL, a, aR, bL, b, bR, cL, cc, cR);
        B[r * NC + c] = w;
        if (own_c && r >= kk && r < kk + th_own) cnt += __popc(w);
        aL = bL; a = b; aR = bR;
        bL = cL; b = cc; bR = cR;
      }
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if (lane == 0 && cnt) atomicAdd(&spop[g - 1], cnt);
    __syncthreads();
    uint32_t *tmp = A; A = B; B = tmp;
  }
  if (tid < kk && spop[tid]) atomicAdd(&pop[tid], spop[tid]);
  // write back the owned words, one warp per row
  if (VEC) {
    // lane L writes cells 4(L%8)..+3 of word L/8 of each 4-word group
    const int sub = lane >> 3, quad = (lane & 7) * 4;
    for (int r = warp; r < th_own; r += nwarps) {
      const uint32_t *src = A + (r + kk) * NC + 1;
      int32_t *dst = next + (size_t)(row0 + r) * p.n0 + (size_t)col0 * 32 + quad;
      for (int c0 = 0; c0 < tw_own; c0 += 16) {
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          const int cw = c0 + 4 * g + sub;
          if (cw < tw_own) {
            const uint32_t w = src[cw] >> quad;
            *reinterpret_cast<int4 *>(dst + (size_t)cw * 32) =
                make_int4((int)(w & 1u), (int)((w >> 1) & 1u), (int)((w >> 2) & 1u),
                          (int)((w >> 3) & 1u));
          }
        }
      }
    }
  } else {
    // lane i writes bit i of each word
    for (int r = warp; r < th_own; r += nwarps) {
      const uint32_t *src = A + (r + kk) * NC + 1;
      int32_t *dst = next + (size_t)(row0 + r) * p.n0 + (size_t)col0 * 32 + lane;
      for (int c0 = 0; c0 < tw_own; c0 += 4) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int c = c0 + j;
          if (c < tw_own) dst[(size_t)c * 32] = (int32_t)((src[c] >> lane) & 1u);
        }
      }
    }
  }
}

// Row sums used by the sliding-window update: horizontal full-adder of the
// three cells W, C, E of every bit position (f1 ones, f2 twos) and
// half-adder of W, E (h1, h2), for one 32-cell word.
struct RowSums {
  uint32_t raw, f1, f2, h1, h2;
};

__device__ __forceinline__ RowSums row_sums(uint32_t left, uint32_t w, uint32_t right) {
  const uint32_t W = __funnelshift_l(left, w, 1), E = __funnelshift_r(w, right, 1);
  RowSums r;
  r.raw = w;
  r.f1 = W ^ w ^ E;
  r.f2 = (W & w) | (E & (W ^ w));
  r.h1 = W ^ E;
  r.h2 = W & E;
  return r;
}

// next state of the middle row b from the sums of rows a (above), b, c:
// num = s0 + 2*(u + k0) with u = a2 + b2 + c2; alive' = (num==3) | (b & num==2)
// = (u + k0 == 1) & (s0 | b) = ~u2 & (u1 ^ k0) & (s0 | b).
__device__ __forceinline__ uint32_t life_from_sums(const RowSums &a, const RowSums &b,
                                                   const RowSums &c) {
  const uint32_t s0 = a.f1 ^ b.h1 ^ c.f1;
  const uint32_t k0 = (a.f1 & b.h1) | (c.f1 & (a.f1 ^ b.h1));
  const uint32_t u1 = a.f2 ^ b.h2 ^ c.f2;
  const uint32_t u2 = (a.f2 & b.h2) | (c.f2 & (a.f2 ^ b.h2));
  return ~u2 & (u1 ^ k0) & (s0 | b.raw);
}

// Whole grid in registers, one packed word per thread: all `gens`
// generations in one launch of one CTA.  The grid is wd = n0 / 32 words
// wide with wd dividing 32, so a warp holds 32 / wd whole rows: lane L has
// word L % wd of row L / wd of its warp.  West and east words come from
// the lanes beside (wrapping within the row), the row sums of the rows
// above and below from lanes L -+ wd; the warp's top and bottom rows take
// them from the neighbouring warps through shared memory (double-buffered
// by generation parity, so one barrier per generation).  Each warp adds its
// population into pop[g] (zeroed by the caller).
__global__ void __launch_bounds__(1024)
life_smallreg_kernel(const int32_t *__restrict__ cur, int32_t *__restrict__ next, int n0, int n1,
                     int gens, uint32_t *__restrict__ pop) {
  __shared__ uint32_t top[2][32][2][32];  // [parity][warp][f1, f2][word]: first row's sums
  __shared__ uint32_t bot[2][32][2][32];  // last row's sums
  const int wd = n0 >> 5, rw = 32 / wd;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int x = lane % wd, r = lane / wd, y = warp * rw + r;
  // pack this thread's word: cells 32x .. 32x + 31 of row y
  const int32_t *src = cur + (size_t)y * n0 + 32 * x;
  uint32_t w = 0;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int4 v = __ldg(reinterpret_cast<const int4 *>(src) + q);
    w |= ((uint32_t)v.x | ((uint32_t)v.y << 1) | ((uint32_t)v.z << 2) | ((uint32_t)v.w << 3))
         << (4 * q);
  }
  const int west = x == 0 ? lane + wd - 1 : lane - 1;
  const int east = x == wd - 1 ? lane - wd + 1 : lane + 1;
  const int up = (lane - wd) & 31, down = (lane + wd) & 31;
  const bool first = r == 0, last = r == rw - 1;
  const int wup = warp == 0 ? nw - 1 : warp - 1, wdown = warp == nw - 1 ? 0 : warp + 1;
  for (int g = 0; g < gens; ++g) {
    const int b = g & 1;
    const RowSums me = row_sums(__shfl_sync(0xffffffffu, w, west), w,
                                __shfl_sync(0xffffffffu, w, east));
    if (first) {
      top[b][warp][0][x] = me.f1;
      top[b][warp][1][x] = me.f2;
    }
    if (last) {
      bot[b][warp][0][x] = me.f1;
      bot[b][warp][1][x] = me.f2;
    }
    RowSums a, c;
    a.f1 = __shfl_sync(0xffffffffu, me.f1, up);
    a.f2 = __shfl_sync(0xffffffffu, me.f2, up);
    c.f1 = __shfl_sync(0xffffffffu, me.f1, down);
    c.f2 = __shfl_sync(0xffffffffu, me.f2, down);
    __syncthreads();
    if (first) {
      a.f1 = bot[b][wup][0][x];
      a.f2 = bot[b][wup][1][x];
    }
    if (last) {
      c.f1 = top[b][wdown][0][x];
      c.f2 = top[b][wdown][1][x];
    }
    w = life_from_sums(a, me, c);
    const uint32_t cnt = __reduce_add_sync(0xffffffffu, __popc(w));
    if (lane == 0 && cnt) atomicAdd(&pop[g], cnt);
  }
  int32_t *dst = next + (size_t)y * n0 + 32 * x;
#pragma unroll
  for (int q = 0; q < 8; ++q)
    reinterpret_cast<int4 *>(dst)[q] =
        make_int4((int)((w >> (4 * q)) & 1u), (int)((w >> (4 * q + 1)) & 1u),
                  (int)((w >> (4 * q + 2)) & 1u), (int)((w >> (4 * q + 3)) & 1u));
}

// Temporal blocking with one lane per packed word: a tile is 32 words wide
// (30 owned + a halo word each side) and th rows tall plus kk halo rows above
// and below.  Each warp sweeps a contiguous band of rows per generation,
// taking the left/right neighbour words from the adjacent lanes and keeping
// the row sums of the previous two rows in registers.
template <bool VEC>
__global__ void __launch_bounds__(256, 8)
life_tb32_kernel(const int32_t *__restrict__ cur, int32_t *__restrict__ next, TbParams p,
                 uint32_t *__restrict__ pop) {
  extern __shared__ uint32_t sm[];
  __shared__ uint32_t spop[32];
  constexpr int NC = 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  const int t = blockIdx.x;
  const int t0 = t % p.nt0, t1 = t / p.nt0;
  const int col0 = t0 * p.tw, row0 = t1 * p.th;
  const int tw_own = min(p.tw, p.wd - col0), th_own = min(p.th, p.n1 - row0);
  const int kk = p.kk;
  const int NR = th_own + 2 * kk;
  const int stride = NC * (p.th + 2 * kk);
  uint32_t *A = sm, *B = sm + stride;
  if (tid < 32) spop[tid] = 0;
  if (VEC)
    pack_rows_vec<4>(cur, p.n0, p.n1, p.wd, row0 - kk, col0 - 1, NC, NR, A, warp, nwarps, lane);
  else
    pack_rows(cur, p.n0, p.n1, p.wd, row0 - kk, col0 - 1, NC, NR, A, warp, nwarps, lane);
  __syncthreads();
  const bool own_c = lane >= 1 && lane <= tw_own;
  for (int g = 1; g <= kk; ++g) {
    const int lo = g, hi = NR - g;
    const int chunk = (hi - lo + nwarps - 1) / nwarps;
    const int rs = lo + warp * chunk, re = min(rs + chunk, hi);
    uint32_t cnt = 0;
    if (rs < re) {
      uint32_t w = A[(rs - 1) * NC + lane];
      RowSums a = row_sums(__shfl_up_sync(0xffffffffu, w, 1) & (lane ? ~0u : 0u), w,
                           __shfl_down_sync(0xffffffffu, w, 1) & (lane < 31 ? ~0u : 0u));
      w = A[rs * NC + lane];
      RowSums b = row_sums(__shfl_up_sync(0xffffffffu, w, 1) & (lane ? ~0u : 0u), w,
                           __shfl_down_sync(0xffffffffu, w, 1) & (lane < 31 ? ~0u : 0u));
      for (int r = rs; r < re; ++r) {
        w = A[(r + 1) * NC + lane];
        const RowSums c = row_sums(__shfl_up_sync(0xffffffffu, w, 1) & (lane ? ~0u : 0u), w,
                                   __shfl_down_sync(0xffffffffu, w, 1) & (lane < 31 ? ~0u : 0u));
        const uint32_t out = life_from_sums(a, b, c);
        B[r * NC + lane] = out;
        if (own_c && r >= kk && r < kk + th_own) cnt += __popc(out);
        a = b;
        b = c;
      }
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if (lane == 0 && cnt) atomicAdd(&spop[g - 1], cnt);
    __syncthreads();
    uint32_t *tmp = A; A = B; B = tmp;
  }
  if (tid < kk && spop[tid]) atomicAdd(&pop[tid], spop[tid]);
  // write back the owned words (block columns 1..tw_own), one warp per row
  if (VEC) {
    const int sub = lane >> 3, quad = (lane & 7) * 4;
    for (int r = warp; r < th_own; r += nwarps) {
      const uint32_t *src = A + (r + kk) * NC + 1;
      int32_t *dst = next + (size_t)(row0 + r) * p.n0 + (size_t)col0 * 32 + quad;
      for (int c0 = 0; c0 < tw_own; c0 += 16) {
#pragma unroll
        for (int gq = 0; gq < 4; ++gq) {
          const int cw = c0 + 4 * gq + sub;
          if (cw < tw_own) {
            const uint32_t wv = src[cw] >> quad;
            *reinterpret_cast<int4 *>(dst + (size_t)cw * 32) =
                make_int4((int)(wv & 1u), (int)((wv >> 1) & 1u), (int)((wv >> 2) & 1u),
                          (int)((wv >> 3) & 1u));
          }
        }
      }
    }
  } else {
    for (int r = warp; r < th_own; r += nwarps) {
      const uint32_t *src = A + (r + kk) * NC + 1;
      int32_t *dst = next + (size_t)(row0 + r) * p.n0 + (size_t)col0 * 32 + lane;
      for (int c = 0; c < tw_own; ++c) dst[(size_t)c * 32] = (int32_t)((src[c] >> lane) & 1u);
    }
  }
}

// Register-resident temporal blocking.  A block is NW warps x R rows of 32
// packed words (30 owned + halo word each side); warp w keeps rows
// [wR, wR+R) in registers for all kk generations and trades only its first
// and last row with the neighbouring warps through shared memory, once per
// generation.  Rows are not shrunk per generation: the stale front from the
// block's outer rows and columns moves one cell per generation and never
// reaches the owned rows [kk, kk + th_own) and words 1..tw_own.
template <int R, int NW, bool VEC>
__global__ void __launch_bounds__(NW * 32, (NW >= 16 ? 2 : 4))
life_reg_kernel(const int32_t *__restrict__ cur, int32_t *__restrict__ next, TbParams p,
                uint32_t *__restrict__ pop) {
  constexpr int NC = 32, NR = R * NW;
  extern __shared__ uint32_t A[];  // NR x NC packed words
  __shared__ uint32_t ex[2][NW][2][NC];
  __shared__ uint32_t spop[32];
  __shared__ int4 nib[16];  // nibble -> its four cells
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid < 16) nib[tid] = make_int4(tid & 1, (tid >> 1) & 1, (tid >> 2) & 1, (tid >> 3) & 1);
  const int t = blockIdx.x;
  const int t0 = t % p.nt0, t1 = t / p.nt0;
  // tiles split the grid evenly (sizes differ by at most one word / row)
  const int col0 = (int)((long long)t0 * p.wd / p.nt0);
  const int row0 = (int)((long long)t1 * p.n1 / p.nt1);
  const int tw_own = (int)((long long)(t0 + 1) * p.wd / p.nt0) - col0;
  const int th_own = (int)((long long)(t1 + 1) * p.n1 / p.nt1) - row0;
  const int kk = p.kk;
  if (tid < 32) spop[tid] = 0;
  if (VEC)
    pack_rows32(cur, p.n0, p.n1, p.wd, row0 - kk, col0 - 1, NR, A, warp, NW, lane);
  else
    pack_rows(cur, p.n0, p.n1, p.wd, row0 - kk, col0 - 1, NC, NR, A, warp, NW, lane);
  __syncthreads();
  uint32_t rows[R];
#pragma unroll
  for (int i = 0; i < R; ++i) rows[i] = A[(warp * R + i) * NC + lane];
  // owned rows of this warp as a bit mask; owned columns as a lane mask
  uint32_t ownrows = 0;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int gr = warp * R + i - kk;
    if (gr >= 0 && gr < th_own) ownrows |= 1u << i;
  }
  const uint32_t colmask = (lane >= 1 && lane <= tw_own) ? ~0u : 0u;
  // most warps own all their rows or none: those count every row and keep
  // the lane's count only if the lane and the rows are owned (no per-row
  // test); the warps on the block's halo edges test each row
  constexpr uint32_t allrows = R == 32 ? ~0u : ((1u << R) - 1u);
  for (int g = 0; g < kk; ++g) {
    const int b = g & 1;
    ex[b][warp][0][lane] = rows[0];
    ex[b][warp][1][lane] = rows[R - 1];
    __syncthreads();
    const uint32_t up = warp > 0 ? ex[b][warp - 1][1][lane] : 0u;
    const uint32_t down = warp < NW - 1 ? ex[b][warp + 1][0][lane] : 0u;
    RowSums ra = row_sums(__shfl_up_sync(0xffffffffu, up, 1), up,
                          __shfl_down_sync(0xffffffffu, up, 1));
    RowSums rb = row_sums(__shfl_up_sync(0xffffffffu, rows[0], 1), rows[0],
                          __shfl_down_sync(0xffffffffu, rows[0], 1));
    uint32_t cnt = 0;
    if (ownrows == allrows || ownrows == 0u) {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const uint32_t wn = (i + 1 < R) ? rows[i + 1] : down;
        const RowSums rc = row_sums(__shfl_up_sync(0xffffffffu, wn, 1), wn,
                                    __shfl_down_sync(0xffffffffu, wn, 1));
        const uint32_t out = life_from_sums(ra, rb, rc);
        rows[i] = out;
        cnt += __popc(out);
        ra = rb;
        rb = rc;
      }
      cnt &= ownrows == allrows ? colmask : 0u;
    } else {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const uint32_t wn = (i + 1 < R) ? rows[i + 1] : down;
        const RowSums rc = row_sums(__shfl_up_sync(0xffffffffu, wn, 1), wn,
                                    __shfl_down_sync(0xffffffffu, wn, 1));
        const uint32_t out = life_from_sums(ra, rb, rc);
        rows[i] = out;
        if (ownrows & (1u << i)) cnt += __popc(out & colmask);
        ra = rb;
        rb = rc;
      }
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    if (lane == 0 && cnt) atomicAdd(&spop[g], cnt);
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < R; ++i) A[(warp * R + i) * NC + lane] = rows[i];
  __syncthreads();
  if (tid < kk && spop[tid]) atomicAdd(&pop[tid], spop[tid]);
  const int sub = lane >> 3, quad = (lane & 7) * 4;
  for (int r = warp; r < th_own; r += NW) {
    const uint32_t *src = A + (r + kk) * NC + 1;
    int32_t *dst = next + (size_t)(row0 + r) * p.n0 + (size_t)col0 * 32;
    if (VEC) {
      // four cells of a word per lane, as the four cells of a nibble
      for (int c0 = 0; c0 < tw_own; c0 += 16) {
#pragma unroll
        for (int gq = 0; gq < 4; ++gq) {
          const int cw = c0 + 4 * gq + sub;
          if (cw < tw_own)
            *reinterpret_cast<int4 *>(dst + (size_t)cw * 32 + quad) =
                nib[(src[cw] >> quad) & 15u];
        }
      }
    } else {
      for (int c = 0; c < tw_own; ++c)
        dst[(size_t)c * 32 + lane] = (int32_t)((src[c] >> lane) & 1u);
    }
  }
}

// Warp-specialised persistent variant of the register-resident kernel: one
// CTA per SM walks its share of the tiles through a three-stage pipeline
// over three shared-memory tile buffers.  In stage s, producer warps pack
// tile s, consumer warps advance tile s-1 by kk generations in registers
// (edge rows traded through shared memory behind a named barrier that only
// the consumers use), and store warps write tile s-2 back, so loads,
// compute and stores of consecutive tiles overlap.  One __syncthreads ends
// every stage; there are no spin waits.
// whether a warp-specialised variant has room for its producers' staged rows
// (2 x 4 KB each) beside its three tile buffers
template <int R, int NWC, int NWP>
__host__ __device__ constexpr bool kStagedPack() {
  return 3 * 4 * 32 * R * NWC + 8192 * NWP <= 212992;
}

// TMA (the tile's rows arrive by tensor copies): producer warps pack from
// 4 KB row boxes (32 cells x 32 words x 1 row of the grid viewed as cells x
// words x rows, 128-byte swizzle) that land in NS slots per warp, complete
// on an mbarrier per slot and are issued NS - 1 boxes ahead of the row being
// packed.  Each lane packs one whole word from
// eight 16-byte chunks of its 128-byte line (the swizzle puts chunk j of
// line L at j ^ (L mod 8), so the warp's loads hit every bank once).  The box reads
// zeros outside the grid; in the first and last tile columns the one halo
// word that wraps around (word n0/32 - 1 left of word 0, word 0 right of
// the last word) comes in as a second, one-word box (`tpatch`, no swizzle)
// on the same mbarrier.  Words further out stay zero: with at most 32
// generations per launch their error front never reaches an owned word.
// Waits are bounded (tma::mbar_wait raises *err).
// PS: consumer warps synchronise each generation with their two neighbours
// only (an mbarrier per warp and buffer parity, signalled once the warp's
// boundary rows are written), instead of a barrier over all consumers
template <int R, int NWC, int NWP, int NWS, bool TMA = false, int NS = 2, bool PS = false>
__global__ void __launch_bounds__((NWC + NWP + NWS) * 32, 1)
life_ws_kernel(const int32_t *__restrict__ cur, int32_t *__restrict__ next, TbParams p,
               uint32_t *__restrict__ pop, const __grid_constant__ CUtensorMap tmap,
               const __grid_constant__ CUtensorMap tpatch, uint32_t *err) {
  constexpr int NC = 32, NR = R * NWC;
  extern __shared__ __align__(1024) uint32_t buf[];  // 3 x NR x NC packed words
  __shared__ uint32_t ex[2][NWC][2][NC];
  __shared__ uint32_t spop[32];
  __shared__ int4 nib[16];  // nibble -> its four cells
  __shared__ uint64_t bars[NWP][NS];
  __shared__ uint64_t cbar[PS ? NWC : 1][2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid < 16) nib[tid] = make_int4(tid & 1, (tid >> 1) & 1, (tid >> 2) & 1, (tid >> 3) & 1);
  const int kk = p.kk;
  const int ntiles = p.nt0 * p.nt1;
  const int m = ntiles > (int)blockIdx.x ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  if (tid < 32) spop[tid] = 0;
  if (TMA && tid < NS * NWP) {
    tma::mbar_init(&bars[tid / NS][tid % NS], 1);
    tma::fence_mbar_init();
  }
  if (PS && tid < 2 * NWC) tma::mbar_init(&cbar[tid >> 1][tid & 1], 1);
  // consumer generations so far (all tiles): generation G exchanges through
  // buffer G & 1, and is use G >> 1 of that buffer's mbarriers
  uint32_t G = 0;
  __syncthreads();
  constexpr int NWT = NWC + NWP + NWS;
  // write back the owned words of tile t from shared-memory buffer A, by
  // warps sw .. of nsw
  auto store_tile = [&](int t, const uint32_t *A, int sw, int nsw) {
    const int col0 = (t % p.nt0) * p.tw, row0 = (t / p.nt0) * p.th;
    const int tw_own = min(p.tw, p.wd - col0), th_own = min(p.th, p.n1 - row0);
    const int sub = lane >> 3, quad = (lane & 7) * 4;
    for (int r = sw; r < th_own; r += nsw) {
      const uint32_t *src = A + (r + kk) * NC + 1;
      int32_t *dst = next + (size_t)(row0 + r) * p.n0 + (size_t)col0 * 32 + quad;
      for (int c0 = 0; c0 < tw_own; c0 += 16) {
#pragma unroll
        for (int gq = 0; gq < 4; ++gq) {
          const int cw = c0 + 4 * gq + sub;
          if (cw < tw_own)
            *reinterpret_cast<int4 *>(dst + (size_t)cw * 32) = nib[(src[cw] >> quad) & 15u];
        }
      }
    }
  };
  auto pack_tile = [&](int s, int pw, int npw) {
    const int t = blockIdx.x + s * gridDim.x;
    const int col0 = (t % p.nt0) * p.tw, row0 = (t / p.nt0) * p.th;
    pack_rows32(cur, p.n0, p.n1, p.wd, row0 - kk, col0 - 1, NR, buf + (s % 3) * NR * NC, pw,
                npw, lane);
  };
  // TMA slots: after the three tile buffers, 1024-byte aligned (the
  // swizzle's period), NS 4 KB slots per producer warp, then NS 128-byte
  // slots per producer warp for the wrapped halo word
  unsigned char *slots = nullptr, *patches = nullptr;
  if (TMA) {
    unsigned char *after = reinterpret_cast<unsigned char *>(buf + 3 * NR * NC);
    slots = after + ((1024u - (tma::smem_addr(after) & 1023u)) & 1023u);
    patches = slots + (size_t)NWP * NS * 4096;
  }
  // rows this producer warp has packed so far; its rows run pw, pw + NWP,
  // ... of tile 1, then of tile 2, ..., and box q of that sequence goes
  // into slot q mod NS
  uint32_t seq = 0;
  // lane whose word wraps around in tile column col0 (-1: none): lane 0
  // holds word -1 in the first column, lane wd - col0 + 1 word wd in the last
  auto wrap_lane = [&](int col0) {
    if (col0 == 0) return 0;
    const int sr = p.wd - col0 + 1;
    return sr <= 31 ? sr : -1;
  };
  auto row_issue = [&](int s, int r, uint32_t q) {
    const int t = blockIdx.x + s * gridDim.x;
    const int col0 = (t % p.nt0) * p.tw, row0 = (t / p.nt0) * p.th;
    int gy = (row0 - kk + r) % p.n1;
    if (gy < 0) gy += p.n1;
    if (lane == 0) {
      const int pw = warp - NWC;
      const int slot = pw * NS + (int)(q % NS);
      uint64_t *bar = &bars[pw][q % NS];
      const int wl = wrap_lane(col0);
      tma::mbar_arrive_expect_tx(bar, wl >= 0 ? 4096 + 128 : 4096);
      tma::load_3d(slots + (size_t)slot * 4096, &tmap, 0, col0 - 1, gy, bar);
      if (wl >= 0)
        tma::load_3d(patches + (size_t)slot * 128, &tpatch, 0, wl == 0 ? p.wd - 1 : 0, gy, bar);
    }
  };
  auto row_pack = [&](int s, int r, uint32_t q) {
    const int t = blockIdx.x + s * gridDim.x;
    const int col0 = (t % p.nt0) * p.tw;
    const int pw = warp - NWC;
    const int slot = pw * NS + (int)(q % NS);
    tma::mbar_wait(&bars[pw][q % NS], (q / NS) & 1, err);
    const bool patched = lane == wrap_lane(col0);
    const unsigned char *line =
        patched ? patches + (size_t)slot * 128 : slots + (size_t)slot * 4096 + lane * 128;
    const int x7 = patched ? 0 : (lane & 7);
    uint32_t w = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int4 c = *reinterpret_cast<const int4 *>(line + ((j ^ x7) << 4));
      w += ((uint32_t)c.x << (4 * j)) + ((uint32_t)c.y << (4 * j + 1)) +
           ((uint32_t)c.z << (4 * j + 2)) + ((uint32_t)c.w << (4 * j + 3));
    }
    buf[(s % 3) * NR * NC + r * NC + lane] = w;
    // the slot's reads are done before the next box into it is issued
    tma::fence_proxy_async();
    __syncwarp();
  };
  // the producers' staging rows follow the three tile buffers
  int4 *stage = reinterpret_cast<int4 *>(buf + 3 * NR * NC);
  auto pack_tile_async = [&](int s, int pw) {
    const int t = blockIdx.x + s * gridDim.x;
    const int col0 = (t % p.nt0) * p.tw, row0 = (t / p.nt0) * p.th;
    pack_rows32_async(cur, p.n0, p.n1, p.wd, row0 - kk, col0 - 1, NR, buf + (s % 3) * NR * NC,
                      pw, NWP, lane, stage + pw * 512);
  };
  // Stage 0 only packs and stage m + 1 only stores: there every warp of the
  // block takes part; in stage m the producers, with no tile left to pack,
  // help the store warps.
  for (int s = 0; s < m + 2; ++s) {
    if (s == 0) {
      if (m > 0) pack_tile(0, warp, NWT);
    } else if (s == m + 1) {
      if (m > 0) store_tile(blockIdx.x + (s - 2) * gridDim.x, buf + ((s - 2) % 3) * NR * NC, warp, NWT);
    } else if (warp < NWC) {
      {
        // consumers: advance tile s-1
        const int t = blockIdx.x + (s - 1) * gridDim.x;
        const int col0 = (t % p.nt0) * p.tw, row0 = (t / p.nt0) * p.th;
        const int tw_own = min(p.tw, p.wd - col0), th_own = min(p.th, p.n1 - row0);
        uint32_t *A = buf + ((s - 1) % 3) * NR * NC;
        uint32_t rows[R];
#pragma unroll
        for (int i = 0; i < R; ++i) rows[i] = A[(warp * R + i) * NC + lane];
        uint32_t ownrows = 0;
#pragma unroll
        for (int i = 0; i < R; ++i) {
          const int gr = warp * R + i - kk;
          if (gr >= 0 && gr < th_own) ownrows |= 1u << i;
        }
        const uint32_t colmask = (lane >= 1 && lane <= tw_own) ? ~0u : 0u;
        for (int g = 0; g < kk; ++g) {
          const int b = PS ? (int)(G & 1u) : (g & 1);
          ex[b][warp][0][lane] = rows[0];
          ex[b][warp][1][lane] = rows[R - 1];
          if (PS) {
            // A neighbour is at most one use ahead on a buffer: to arrive
            // again it must first see this warp's next generation.  It
            // reads a buffer before it signals the next generation, so
            // this warp's rewrite two generations on cannot overtake it.
            __syncwarp();
            if (lane == 0) tma::mbar_arrive(&cbar[warp][b]);
            const uint32_t par = (G >> 1) & 1u;
            if (warp > 0) tma::mbar_wait(&cbar[warp - 1][b], par, err);
            if (warp < NWC - 1) tma::mbar_wait(&cbar[warp + 1][b], par, err);
            ++G;
          } else {
            asm volatile("bar.sync 1, %0;" ::"r"(NWC * 32) : "memory");
          }
          const uint32_t up = warp > 0 ? ex[b][warp - 1][1][lane] : 0u;
          const uint32_t down = warp < NWC - 1 ? ex[b][warp + 1][0][lane] : 0u;
          RowSums ra = row_sums(__shfl_up_sync(0xffffffffu, up, 1), up,
                                __shfl_down_sync(0xffffffffu, up, 1));
          RowSums rb = row_sums(__shfl_up_sync(0xffffffffu, rows[0], 1), rows[0],
                                __shfl_down_sync(0xffffffffu, rows[0], 1));
          uint32_t cnt = 0;
          constexpr uint32_t allrows = R == 32 ? ~0u : ((1u << R) - 1u);
          if (ownrows == allrows || ownrows == 0u) {
#pragma unroll
            for (int i = 0; i < R; ++i) {
              const uint32_t wn = (i + 1 < R) ? rows[i + 1] : down;
              const RowSums rc = row_sums(__shfl_up_sync(0xffffffffu, wn, 1), wn,
                                          __shfl_down_sync(0xffffffffu, wn, 1));
              const uint32_t out = life_from_sums(ra, rb, rc);
              rows[i] = out;
              cnt += __popc(out);
              ra = rb;
              rb = rc;
            }
            cnt &= ownrows == allrows ? colmask : 0u;
          } else {
#pragma unroll
            for (int i = 0; i < R; ++i) {
              const uint32_t wn = (i + 1 < R) ? rows[i + 1] : down;
              const RowSums rc = row_sums(__shfl_up_sync(0xffffffffu, wn, 1), wn,
                                          __shfl_down_sync(0xffffffffu, wn, 1));
              const uint32_t out = life_from_sums(ra, rb, rc);
              rows[i] = out;
              if (ownrows & (1u << i)) cnt += __popc(out & colmask);
              ra = rb;
              rb = rc;
            }
          }
          cnt = __reduce_add_sync(0xffffffffu, cnt);
          if (lane == 0 && cnt) atomicAdd(&spop[g], cnt);
        }
#pragma unroll
        for (int i = 0; i < R; ++i) A[(warp * R + i) * NC + lane] = rows[i];
      }
    } else if (warp < NWC + NWP) {
      if (s < m)
        if (TMA) {
          // rows pw, pw + NWP, ... of tile s, NS - 1 boxes ahead (the first
          // rows of tile s + 1 follow the last of tile s); a slot is issued
          // into only after the row it held was packed
          const int pw = warp - NWC;
          if (s == 1) {  // the sequence's first NS - 1 boxes
            int nr = pw, ns = 1;
            for (int k = 0; k < NS - 1 && ns < m; ++k) {
              row_issue(ns, nr, (uint32_t)k);
              nr += NWP;
              if (nr >= NR) {
                nr = pw;
                ++ns;
              }
            }
          }
          for (int r = pw; r < NR; r += NWP) {
            // the row NS - 1 places further on in the sequence
            int nr = r, ns = s;
#pragma unroll
            for (int k = 0; k < NS - 1; ++k) {
              nr += NWP;
              if (nr >= NR) {
                nr = pw;
                ++ns;
              }
            }
            if (ns < m) row_issue(ns, nr, seq + NS - 1);
            row_pack(s, r, seq);
            ++seq;
          }
        } else if (kStagedPack<R, NWC, NWP>())
          pack_tile_async(s, warp - NWC);
        else
          pack_tile(s, warp - NWC, NWP);
      else if (s >= 2)  // s == m
        store_tile(blockIdx.x + (s - 2) * gridDim.x, buf + ((s - 2) % 3) * NR * NC, warp - NWC,
                   NWP + NWS);
    } else if (s >= 2) {
      // store warps: write back tile s - 2
      const bool helped = s == m;
      store_tile(blockIdx.x + (s - 2) * gridDim.x, buf + ((s - 2) % 3) * NR * NC,
                 helped ? warp - NWC : warp - NWC - NWP, helped ? NWP + NWS : NWS);
    }
    __syncthreads();
  }
  if (tid < kk && spop[tid]) atomicAdd(&pop[tid], spop[tid]);
}

__global__ void life_fill_kernel(int32_t *cell, int n0, int n1, int ms0, int lm,
                                 uint64_t seed_mix, uint64_t thr) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  const size_t total = (size_t)n0 * n1;
  if (i >= total) return;
  const size_t y = i / n0, x = i - y * n0;
  const uint64_t h = mix64(seed_mix + (uint64_t)i * 0x9E3779B97F4A7C15ULL);
  cell[(y + lm) * ms0 + (x + lm)] = ((h >> 11) < thr) ? 1 : 0;
}

__global__ void life_finalize_kernel(LifeScalars *s, const uint32_t *pop, int n) {
  s->population = (int32_t)pop[n - 1];
  s->generation = (int32_t)((uint32_t)s->generation + (uint32_t)n);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// Grids up to this many packed words run all generations in one CTA; larger
// ones spread over every SM with the temporally blocked tiles.
static const int kSmallMaxWords = 4096;

static om_status life_reserve(Handle *h, int kernel_id, int n) {
  (void)kernel_id;
  LifeState *st = life_state(h);
  if (n <= st->pop_cap) return OM_OK;
  int cap = std::max(n, 1024);
  uint32_t *p = nullptr;
  if (cudaMalloc(&p, (size_t)cap * sizeof(uint32_t)) != cudaSuccess) {
    cudaGetLastError();
    set_error("Life: cannot allocate the population history");
    return OM_ERR_NOMEM;
  }
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  if (st->d_pop) cudaFree(st->d_pop);
  st->d_pop = p;
  st->pop_cap = cap;
  return OM_OK;
}

static om_status life_init(Handle *h, int n) {
  (void)n;
  Array &a = h->arrays[0];
  OM_CUDA_CHECK(cudaMemsetAsync(a.d(), 0, a.count * sizeof(int32_t), h->stream));
  OM_CUDA_CHECK(cudaMemsetAsync(h->d_scalars, 0, sizeof(LifeScalars), h->stream));
  life_state(h)->binary = true;
  life_state(h)->last_n = 0;
  return OM_OK;
}

// Register-resident kernel variants: R rows per warp x NW warps per block.
struct RegVariant {
  int R, NW;
};
static const RegVariant kRegVariants[] = {{16, 8}, {24, 8}, {16, 16}, {32, 8}, {24, 16}, {32, 16}};
static const int kNumRegVariants = 6;

template <bool VEC>
static cudaError_t launch_reg(int v, const int32_t *cur, int32_t *next, const TbParams &p,
                              uint32_t *pop, cudaStream_t s) {
  const RegVariant rv = kRegVariants[v];
  const size_t smem = sizeof(uint32_t) * 32 * rv.R * rv.NW;
  void (*k)(const int32_t *, int32_t *, TbParams, uint32_t *) = nullptr;
  switch (v) {
    case 0: k = life_reg_kernel<16, 8, VEC>; break;
    case 1: k = life_reg_kernel<24, 8, VEC>; break;
    case 2: k = life_reg_kernel<16, 16, VEC>; break;
    case 3: k = life_reg_kernel<32, 8, VEC>; break;
    case 4: k = life_reg_kernel<24, 16, VEC>; break;
    default: k = life_reg_kernel<32, 16, VEC>; break;
  }
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  k<<<p.nt0 * p.nt1, rv.NW * 32, smem, s>>>(cur, next, p, pop);
  return cudaGetLastError();
}

// warp-specialised variants: R rows x NWC consumer warps, NWP producer and
// NWS store warps, one CTA per SM
struct WsVariant {
  int R, NWC, NWP, NWS;
  bool tma;  // producers take their rows by TMA
  int ns;    // TMA slots per producer warp
  bool ps;   // consumers synchronise with their neighbours only
};
static const WsVariant kWsVariants[] = {
    {24, 16, 8, 8, false, 0}, {16, 16, 8, 8, false, 0}, {24, 16, 12, 4, false, 0},
    {20, 16, 8, 8, false, 0}, {20, 16, 8, 8, true, 2},  {24, 16, 8, 8, true, 2},
    {20, 16, 4, 12, true, 4}, {20, 16, 6, 10, true, 3}, {24, 16, 4, 12, true, 4},
    {21, 16, 8, 8, true, 2},  {22, 16, 8, 8, true, 2},  {21, 16, 8, 8, false, 0},
    {22, 16, 8, 8, false, 0}, {23, 16, 8, 8, true, 2},  {22, 16, 8, 8, true, 2, true},
    {20, 16, 8, 8, true, 2, true}};
static const int kNumWsVariants = 16;
// the variant the automatic choice takes when TMA serves the grid (rows of
// at least 32 words; fastest on GB300 at 16384^2: 22 rows per consumer warp
// give 990 tiles, at most 7 per SM, where 20 rows give 1098, at most 8),
// else the staged-copy one
static const int kAutoWsVariantTma = 10;
static const int kAutoWsVariant = 3;

// `tmap`, `tpatch`: the tensor maps of `cur` for the TMA variants (ignored
// by the others); at most `ctas` persistent CTAs
static cudaError_t launch_ws(int v, const int32_t *cur, int32_t *next, const TbParams &p,
                             uint32_t *pop, int ctas, const CUtensorMap &tmap,
                             const CUtensorMap &tpatch, uint32_t *err, cudaStream_t s) {
  const WsVariant wv = kWsVariants[v];
  size_t smem = sizeof(uint32_t) * 3 * 32 * wv.R * wv.NWC;
  if (wv.tma) {
    // three tile buffers, alignment slack, ns 4 KB TMA slots and ns
    // 128-byte wrapped-word slots per producer warp
    smem += 1024 + (size_t)(4096 + 128) * wv.ns * wv.NWP;
  } else if (3 * 4 * 32 * wv.R * wv.NWC + 8192 * wv.NWP <= 212992) {
    // three tile buffers, then two staged rows (2 x 4 KB) per producer warp
    smem += sizeof(int4) * 512 * wv.NWP;
  }
  void (*k)(const int32_t *, int32_t *, TbParams, uint32_t *, const CUtensorMap,
            const CUtensorMap, uint32_t *) = nullptr;
  switch (v) {
    case 0: k = life_ws_kernel<24, 16, 8, 8>; break;
    case 1: k = life_ws_kernel<16, 16, 8, 8>; break;
    case 2: k = life_ws_kernel<24, 16, 12, 4>; break;
    case 3: k = life_ws_kernel<20, 16, 8, 8>; break;
    case 4: k = life_ws_kernel<20, 16, 8, 8, true, 2>; break;
    case 5: k = life_ws_kernel<24, 16, 8, 8, true, 2>; break;
    case 6: k = life_ws_kernel<20, 16, 4, 12, true, 4>; break;
    case 7: k = life_ws_kernel<20, 16, 6, 10, true, 3>; break;
    case 8: k = life_ws_kernel<24, 16, 4, 12, true, 4>; break;
    case 9: k = life_ws_kernel<21, 16, 8, 8, true, 2>; break;
    case 10: k = life_ws_kernel<22, 16, 8, 8, true, 2>; break;
    case 11: k = life_ws_kernel<21, 16, 8, 8>; break;
    case 12: k = life_ws_kernel<22, 16, 8, 8>; break;
    case 13: k = life_ws_kernel<23, 16, 8, 8, true, 2>; break;
    case 14: k = life_ws_kernel<22, 16, 8, 8, true, 2, true>; break;
    default: k = life_ws_kernel<20, 16, 8, 8, true, 2, true>; break;
  }
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  const int ntiles = p.nt0 * p.nt1;
  const int grid = ntiles < ctas ? ntiles : ctas;
  k<<<grid, (wv.NWC + wv.NWP + wv.NWS) * 32, smem, s>>>(cur, next, p, pop, tmap, tpatch, err);
  return cudaGetLastError();
}

// Resident blocks per SM of a register variant (queried once per device;
// handles on other host threads may ask at the same time).
static int reg_occupancy(int device, int v, bool vec) {
  static std::atomic<int> cache[64][kNumRegVariants][2];
  if (device < 0 || device >= 64) return 1;
  std::atomic<int> &c = cache[device][v][vec ? 1 : 0];
  const int known = c.load(std::memory_order_relaxed);
  if (known) return known;
  const RegVariant rv = kRegVariants[v];
  const size_t smem = sizeof(uint32_t) * 32 * rv.R * rv.NW;
  void (*k)(const int32_t *, int32_t *, TbParams, uint32_t *) = nullptr;
  switch (v) {
    case 0: k = vec ? life_reg_kernel<16, 8, true> : life_reg_kernel<16, 8, false>; break;
    case 1: k = vec ? life_reg_kernel<24, 8, true> : life_reg_kernel<24, 8, false>; break;
    case 2: k = vec ? life_reg_kernel<16, 16, true> : life_reg_kernel<16, 16, false>; break;
    case 3: k = vec ? life_reg_kernel<32, 8, true> : life_reg_kernel<32, 8, false>; break;
    case 4: k = vec ? life_reg_kernel<24, 16, true> : life_reg_kernel<24, 16, false>; break;
    default: k = vec ? life_reg_kernel<32, 16, true> : life_reg_kernel<32, 16, false>; break;
  }
  cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, rv.NW * 32, smem) != cudaSuccess || n < 1) {
    cudaGetLastError();
    n = 1;
  }
  c.store(n, std::memory_order_relaxed);
  return n;
}

// Launch plan for the register kernel: the variant and tile grid (nt0 x nt1,
// tiles split evenly).  The kernel is issue-bound and a warp issues for all
// 32 lanes however many words its tile owns, so a block costs its rows
// (NR) whatever its width.  The plan minimises the rows the busiest SM
// issues (ceil(tiles / SMs) x NR), then the rows issued in all (tiles x
// NR).  The 32-row variants need more than the 64 registers a thread has
// at their occupancy and spill: the plan leaves them out.  Returns the
// variant.
static int reg_plan(int device, bool vec, int wd, int n1, int kk, int *nt0_out, int *nt1_out) {
  const int sms = sm_count(device);
  double best_cost = 1e300, best_work = 1e300;
  int best_v = 1, best0 = (wd + 29) / 30, best1 = 1;
  for (int v = 0; v < kNumRegVariants; ++v) {
    if (kRegVariants[v].R > 24) continue;
    const int NR = kRegVariants[v].R * kRegVariants[v].NW;
    const int thm = NR - 2 * kk;
    if (thm < 8) continue;
    if (reg_occupancy(device, v, vec) < 1) continue;
    const int nt0min = (wd + 29) / 30;
    const int nt1min = (n1 + thm - 1) / thm;
    for (int nt0 = nt0min; nt0 <= nt0min + 2 && nt0 <= wd; ++nt0)
      for (int nt1 = nt1min; nt1 <= nt1min + 24 && nt1 <= n1; ++nt1) {
        const long long tiles = (long long)nt0 * nt1;
        const double cost = (double)((tiles + sms - 1) / sms) * NR;
        const double work = (double)tiles * NR;
        if (cost < best_cost - 1e-9 || (cost < best_cost + 1e-9 && work < best_work - 1e-9)) {
          best_cost = cost;
          best_work = work;
          best_v = v;
          best0 = nt0;
          best1 = nt1;
        }
      }
  }
  *nt0_out = best0;
  *nt1_out = best1;
  return best_v;
}

// register variant for kk generations: the smallest block whose owned rows
// (block rows - 2kk) reach the requested tile height (default 320, the
// 24-row x 16-warp block at depth 32: fastest in the GB300 tile sweep)
static int reg_variant(int kk, int want_th) {
  const int want = want_th > 0 ? want_th : 320;
  int best = -1;
  for (int v = 0; v < kNumRegVariants; ++v) {
    const int th = kRegVariants[v].R * kRegVariants[v].NW - 2 * kk;
    if (th >= want) { best = v; break; }
    if (th >= 1) best = v;
  }
  return best < 0 ? kNumRegVariants - 1 : best;
}

// Tile choice: tile_w 0 (default) selects the register-resident kernel,
// 30 the one-lane-per-word shared-memory kernel, other widths the general
// tile kernel.  Depth defaults to 32 generations per launch.
static bool life_pick_tiles(Handle *h, TbParams &p) {
  LifeState *st = life_state(h);
  const bool lane_per_word = st->tile_w == 0 || st->tile_w == 30;
  p.kk = st->depth > 0 ? std::min(st->depth, 32) : 32;
  p.tw = lane_per_word ? 30 : st->tile_w;
  p.th = st->tile_h > 0 ? st->tile_h : 128;
  p.tw = std::min(p.tw, p.wd);
  p.th = std::min(p.th, p.n1);
  return lane_per_word;
}

static size_t tb_smem_bytes(const TbParams &p, bool lane_per_word) {
  const int nc = lane_per_word ? 32 : p.tw + 2;
  return 2 * sizeof(uint32_t) * (size_t)nc * (p.th + 2 * p.kk);
}

static om_status launch_general(Handle *h, uint32_t *pop) {
  Array &a = h->arrays[0];
  const int ms0 = (int)h->memory_size(0), ms1 = (int)h->memory_size(1);
  const int tiles_x = (ms0 + 31) / 32;
  const size_t blocks = (size_t)tiles_x * ((ms1 + 7) / 8);
  dim3 block(32, 8);
  cudaEvent_t ev = prof_begin(h);
  if (h->cyclic)
    life_general_kernel<true><<<(unsigned)blocks, block, 0, h->stream>>>(
        (const int32_t *)a.d(), (int32_t *)a.d_next(), ms0, ms1, 0, tiles_x, pop);
  else
    life_general_kernel<false><<<(unsigned)blocks, block, 0, h->stream>>>(
        (const int32_t *)a.d(), (int32_t *)a.d_next(), ms0, ms1, h->lower_margin[0],
        tiles_x, pop);
  OM_CUDA_CHECK(cudaGetLastError());
  prof_end(h, ev, "life_general_kernel", (double)h->size[0] * h->size[1]);
  h->launches++;
  a.swap();
  return OM_OK;
}

static om_status life_proceed(Handle *h, int n) {
  LifeState *st = life_state(h);
  if (n > st->pop_cap) {
    set_error("Life: population history not reserved");
    return OM_ERR_STATE;
  }
  Array &a = h->arrays[0];
  OM_CUDA_CHECK(cudaMemsetAsync(st->d_pop, 0, (size_t)n * sizeof(uint32_t), h->stream));
  const int n0 = h->size[0], n1 = h->size[1];
  const bool packed_ok = h->cyclic && (n0 % 32 == 0) && h->cfg.variant == 0;
  int g = 0;
  if (!packed_ok || !st->binary) {
    const int first = packed_ok ? 1 : n;
    for (; g < first; ++g) OM_TRY(launch_general(h, st->d_pop + g));
    st->binary = true;
  }
  if (g < n) {
    const int wd = n0 / 32;
    if (32 % wd == 0 && (n1 * wd) % 32 == 0 && n1 * wd <= 1024 && n1 * wd >= 32) {
      // one packed word per thread of one CTA, in registers
      cudaEvent_t ev = prof_begin(h);
      life_smallreg_kernel<<<1, n1 * wd, 0, h->stream>>>(
          (const int32_t *)a.d(), (int32_t *)a.d_next(), n0, n1, n - g, st->d_pop + g);
      OM_CUDA_CHECK(cudaGetLastError());
      prof_end(h, ev, "life_smallreg_kernel", (double)n0 * n1 * (n - g));
      h->launches++;
      a.swap();
    } else if ((size_t)wd * n1 <= (size_t)kSmallMaxWords) {
      const size_t smem = 2 * sizeof(uint32_t) * (size_t)wd * n1;
      OM_CUDA_CHECK(cudaFuncSetAttribute(life_smallgrid_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
      cudaEvent_t ev = prof_begin(h);
      life_smallgrid_kernel<<<1, 512, smem, h->stream>>>(
          (const int32_t *)a.d(), (int32_t *)a.d_next(), n0, n1, n - g, st->d_pop + g);
      OM_CUDA_CHECK(cudaGetLastError());
      prof_end(h, ev, "life_smallgrid_kernel", (double)n0 * n1 * (n - g));
      h->launches++;
      a.swap();
    } else {
      TbParams p;
      p.n0 = n0; p.n1 = n1; p.wd = wd;
      const bool l32 = life_pick_tiles(h, p);
      const bool reg = st->tile_w == 0;
      const int kmax = p.kk;
      p.nt0 = (p.wd + p.tw - 1) / p.tw;
      p.nt1 = (p.n1 + p.th - 1) / p.th;
      // split the remaining generations into launches of near-equal depth
      const int rem = n - g;
      const int nl = (rem + kmax - 1) / kmax;
      const size_t smem_max = tb_smem_bytes(p, l32);
      const bool vec = h->cfg.life_io != 1;
      auto kern = l32 ? (vec ? life_tb32_kernel<true> : life_tb32_kernel<false>)
                      : (vec ? life_tb_kernel<true> : life_tb_kernel<false>);
      const char *kname = l32 ? "life_tb32_kernel" : "life_tb_kernel";
      if (!reg)
        OM_CUDA_CHECK(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem_max));
      // the packed kernel: life_kernel >= 1 selects the warp-specialised
      // persistent kernel (variant life_kernel - 1); 0 with no tile shape
      // given takes it too on grids of at least 1.5 of its tiles per SM,
      // where it overlaps one tile's loads and stores with another's
      // generations, and the register-resident blocks on smaller grids
      int ws = h->cfg.life_kernel;
      // TMA rows need a grid at least one box (32 words) wide whose buffers
      // the driver describes
      const bool tma_ok = wd >= 32 && life_tmap(st, a.d(), n0, n1) >= 0 &&
                          life_tmap(st, a.d_next(), n0, n1) >= 0;
      if (reg && ws == 0 && st->tile_h == 0) {
        const int av = tma_ok ? kAutoWsVariantTma : kAutoWsVariant;
        const WsVariant wv = kWsVariants[av];
        const int th = std::min(wv.R * wv.NWC - 2 * kmax, n1);
        const long long tiles = (long long)((wd + 29) / 30) * ((n1 + th - 1) / th);
        if (th > 0 && 2 * tiles >= 3LL * sm_count(h->device)) ws = av + 1;
      }
      if (ws >= 1 && kWsVariants[std::min(ws - 1, kNumWsVariants - 1)].tma && !tma_ok) {
        set_error("Life: the TMA kernel variants need rows of at least 1024 cells and a "
                  "tensor map of the grid");
        return OM_ERR_UNSUPPORTED;
      }
      for (int l = 0; l < nl; ++l) {
        const int kk = rem / nl + (l < rem % nl ? 1 : 0);
        p.kk = kk;
        if (reg && ws >= 1) {
          // warp-specialised persistent kernel, variant ws - 1
          const int v = std::min(ws - 1, kNumWsVariants - 1);
          const WsVariant wv = kWsVariants[v];
          TbParams q = p;
          q.tw = std::min(30, wd);
          q.th = std::min(wv.R * wv.NWC - 2 * kk, n1);
          q.nt0 = (wd + q.tw - 1) / q.tw;
          q.nt1 = (n1 + q.th - 1) / q.th;
          cudaEvent_t ev = prof_begin(h);
          const int mi = wv.tma ? life_tmap(st, a.d(), n0, n1) : -1;
          const int ctas = h->cfg.grid_limit > 0
                               ? std::min(h->cfg.grid_limit, sm_count(h->device))
                               : sm_count(h->device);
          cudaError_t e = launch_ws(v, (const int32_t *)a.d(), (int32_t *)a.d_next(), q,
                                    st->d_pop + g, ctas, st->tmap[mi < 0 ? 0 : mi],
                                    st->tpatch[mi < 0 ? 0 : mi],
                                    &((LifeScalars *)h->d_scalars)->wait_error, h->stream);
          if (e != cudaSuccess) {
            set_error(std::string("life_ws_kernel: ") + cudaGetErrorString(e));
            return OM_ERR_CUDA;
          }
          prof_end(h, ev, wv.tma ? "life_ws_tma_kernel" : "life_ws_kernel",
                   (double)n0 * n1 * kk);
          h->launches++;
          a.swap();
          g += kk;
          continue;
        }
        if (reg) {
          TbParams q = p;
          const int v = st->tile_h > 0 ? reg_variant(kk, st->tile_h)
                                       : reg_plan(h->device, vec, wd, n1, kk, &q.nt0, &q.nt1);
          if (st->tile_h > 0) {
            const int thm = std::min(kRegVariants[v].R * kRegVariants[v].NW - 2 * kk, n1);
            q.nt0 = (wd + 29) / 30;
            q.nt1 = (n1 + thm - 1) / thm;
          }
          q.tw = (wd + q.nt0 - 1) / q.nt0;
          q.th = (n1 + q.nt1 - 1) / q.nt1;
          cudaEvent_t ev = prof_begin(h);
          cudaError_t e = vec ? launch_reg<true>(v, (const int32_t *)a.d(), (int32_t *)a.d_next(),
                                                 q, st->d_pop + g, h->stream)
                              : launch_reg<false>(v, (const int32_t *)a.d(),
                                                  (int32_t *)a.d_next(), q, st->d_pop + g,
                                                  h->stream);
          if (e != cudaSuccess) {
            set_error(std::string("life_reg_kernel: ") + cudaGetErrorString(e));
            return OM_ERR_CUDA;
          }
          prof_end(h, ev, "life_reg_kernel", (double)n0 * n1 * kk);
          h->launches++;
          a.swap();
          g += kk;
          continue;
        }
        cudaEvent_t ev = prof_begin(h);
        kern<<<p.nt0 * p.nt1, 256, tb_smem_bytes(p, l32), h->stream>>>(
            (const int32_t *)a.d(), (int32_t *)a.d_next(), p, st->d_pop + g);
        OM_CUDA_CHECK(cudaGetLastError());
        prof_end(h, ev, kname, (double)n0 * n1 * kk);
        h->launches++;
        a.swap();
        g += kk;
      }
    }
  }
  life_finalize_kernel<<<1, 1, 0, h->stream>>>((LifeScalars *)h->d_scalars, st->d_pop, n);
  OM_CUDA_CHECK(cudaGetLastError());
  h->launches++;
  st->last_n = n;
  return OM_OK;
}

static uint64_t life_state_key(Handle *h) { return life_state(h)->binary ? 1 : 0; }

static void life_after_replay(Handle *h, int kernel_id, int n) {
  LifeState *st = life_state(h);
  if (h->kernels[kernel_id].name == "proceed") {
    st->binary = true;
    st->last_n = n;
  } else {
    st->binary = true;
    st->last_n = 0;
  }
}

static void life_restore_key(Handle *h, uint64_t key) { life_state(h)->binary = key != 0; }

// New cell contents came from the host.  The packed kernels need every cell
// in {0, 1}; one read-only pass (HBM speed, a fraction of one generation)
// settles that here, outside any stream capture, so that only grids that do
// hold other values pay for a generation of the general integer kernel.
static void life_array_written(Handle *h, Array *a) {
  LifeState *st = life_state(h);
  st->binary = false;
  const bool packed_ok = h->cyclic && (h->size[0] % 32 == 0) && h->cfg.variant == 0;
  if (!packed_ok || !st->d_flag || h->capturing) return;
  uint32_t bad = 1;
  if (cudaMemsetAsync(st->d_flag, 0, sizeof(uint32_t), h->stream) != cudaSuccess ||
      life_check_cells_into((const int32_t *)a->d(), a->count, st->d_flag, h->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(&bad, st->d_flag, sizeof(bad), cudaMemcpyDeviceToHost, h->stream) !=
          cudaSuccess ||
      cudaStreamSynchronize(h->stream) != cudaSuccess)
    return;  // binary stays false: the general kernel handles any values
  st->binary = bad == 0;
}

static void life_free(Handle *h) {
  LifeState *st = life_state(h);
  if (st) {
    if (st->d_pop) cudaFree(st->d_pop);
    if (st->d_flag) cudaFree(st->d_flag);
    delete st;
  }
  h->impl = nullptr;
}

// Raises *flag when any of the n cells is outside {0, 1}.  128-bit loads when
// the array is 16-byte aligned; a value v is outside {0, 1} iff v & ~1 != 0,
// so the OR of four cells is tested at once.
__global__ void __launch_bounds__(256)
life_check_kernel(const int32_t *__restrict__ cells, size_t n, uint32_t *flag) {
  bool bad = false;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t i0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  size_t tail = 0;
  if ((reinterpret_cast<uintptr_t>(cells) & 15) == 0) {
    const int4 *v = reinterpret_cast<const int4 *>(cells);
    const size_t nv = n / 4;
    for (size_t i = i0; i < nv; i += stride) {
      const int4 c = __ldcs(v + i);
      bad |= ((c.x | c.y | c.z | c.w) & ~1) != 0;
    }
    tail = nv * 4;
  }
  for (size_t i = tail + i0; i < n; i += stride) bad |= (cells[i] & ~1) != 0;
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// Launches the cell-value check on stream s (allocates nothing; *flag must
// be cleared by the caller).
cudaError_t life_check_cells_into(const int32_t *cells, size_t n, uint32_t *flag,
                                  cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const size_t want = (n / 4 + 255) / 256;
  const unsigned grid = (unsigned)std::max<size_t>(1, std::min<size_t>(want, 8 * (size_t)sms));
  life_check_kernel<<<grid, 256, 0, s>>>(cells, n, flag);
  return cudaGetLastError();
}

// One launch of the temporally blocked tile kernel from `cur` into `next`
// (cyclic, width % 32 == 0, 1 <= gens <= 32, cells 0/1), with the default
// 32-word x 64-row tiles.  Allocates nothing; used by the caller-buffer
// entry point in life_noalloc.cu.
cudaError_t life_tb_launch_into(const int32_t *cur, int32_t *next, int n0, int n1, int gens,
                                uint32_t *pop, cudaStream_t s) {
  TbParams p;
  p.n0 = n0; p.n1 = n1; p.wd = n0 / 32;
  p.kk = gens;
  p.tw = std::min(32, p.wd);
  p.th = std::min(64, n1);
  p.nt0 = (p.wd + p.tw - 1) / p.tw;
  p.nt1 = (p.n1 + p.th - 1) / p.th;
  const size_t smem = tb_smem_bytes(p, false);
  cudaError_t e = cudaFuncSetAttribute(life_tb_kernel<false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  life_tb_kernel<false><<<p.nt0 * p.nt1, 256, smem, s>>>(cur, next, p, pop);
  return cudaGetLastError();
}

om_status life_setup(Handle *h) {
  const int lm = h->cyclic ? 0 : 1;  // stencil radius 1 (OMTrans.hs:103-116)
  for (int ax = 0; ax < 2; ++ax) {
    h->lower_margin[ax] = lm;
    h->upper_margin[ax] = lm;
  }
  LifeState *st = new LifeState();
  st->depth = h->cfg.depth;
  st->tile_w = h->cfg.tile_x;
  st->tile_h = h->cfg.tile_y;
  h->impl = st;
  h->impl_free = life_free;
  h->ops.state_key = life_state_key;
  h->ops.after_replay = life_after_replay;
  h->ops.restore_key = life_restore_key;
  h->ops.array_written = life_array_written;
  h->ops.reserve = life_reserve;
  h->ops.after_run = [](Handle *hh) -> om_status {
    LifeScalars *sc = (LifeScalars *)hh->h_scalars;
    if (!sc->wait_error) return OM_OK;
    sc->wait_error = 0;  // cleared on the device by the next upload
    set_error("Life: a kernel's bounded wait for its tensor copies ran out; the cells of "
              "this run are unspecified");
    return OM_ERR_CUDA;
  };
  OM_TRY(alloc_array(h, "cell", sizeof(int32_t)));
  if (cudaMalloc(&st->d_flag, sizeof(uint32_t)) != cudaSuccess) {
    set_error("Life: cannot allocate the cell-value flag");
    return OM_ERR_NOMEM;
  }
  h->scalars.push_back({"population", kInt, offsetof(LifeScalars, population)});
  h->scalars.push_back({"generation", kInt, offsetof(LifeScalars, generation)});
  h->scalar_bytes = sizeof(LifeScalars);
  h->kernels.push_back({"init", life_init});
  h->kernels.push_back({"proceed", life_proceed});
  return OM_OK;
}

}  // namespace om

using namespace om;

extern "C" om_status om_life_fill_random(om_handle H, uint64_t seed, double p) {
  if (!H) { set_error("om_life_fill_random: null handle"); return OM_ERR_ARG; }
  Handle *h = handle_of(H);
  if (h->kind != OM_KIND_LIFE) { set_error("not a Life handle"); return OM_ERR_ARG; }
  if (!(p >= 0.0 && p <= 1.0)) { set_error("p must be in [0,1]"); return OM_ERR_ARG; }
  OM_CUDA_CHECK(cudaSetDevice(h->device));
  Array &a = h->arrays[0];
  OM_CUDA_CHECK(cudaMemsetAsync(a.d(), 0, a.count * sizeof(int32_t), h->stream));
  const uint64_t thr = (uint64_t)floor(p * 9007199254740992.0);
  const size_t total = (size_t)h->size[0] * h->size[1];
  const int block = 256;
  life_fill_kernel<<<(unsigned)((total + block - 1) / block), block, 0, h->stream>>>(
      (int32_t *)a.d(), h->size[0], h->size[1], (int)h->memory_size(0),
      h->lower_margin[0], mix64(seed), thr);
  OM_CUDA_CHECK(cudaGetLastError());
  OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  a.newer = a.host ? Newer::kDevice : Newer::kBoth;
  life_state(h)->binary = true;
  return OM_OK;
}

extern "C" om_status om_life_population_history(om_handle H, int32_t *out, int n,
                                                int *written) {
  if (!H || (!out && n > 0)) { set_error("om_life_population_history: null argument"); return OM_ERR_ARG; }
  Handle *h = handle_of(H);
  if (h->kind != OM_KIND_LIFE) { set_error("not a Life handle"); return OM_ERR_ARG; }
  LifeState *st = life_state(h);
  const int m = std::min(n, st->last_n);
  if (m > 0) {
    OM_CUDA_CHECK(cudaSetDevice(h->device));
    OM_CUDA_CHECK(cudaMemcpyAsync(out, st->d_pop, (size_t)m * sizeof(int32_t),
                                  cudaMemcpyDeviceToHost, h->stream));
    OM_CUDA_CHECK(cudaStreamSynchronize(h->stream));
  }
  if (written) *written = std::max(m, 0);
  return OM_OK;
}

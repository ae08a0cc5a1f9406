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
#include <cmath>
#include <cstring>
#include <string>

#include "om_internal.cuh"

namespace om {

struct LifeScalars {  // device/host scalar block
  int32_t population;
  int32_t generation;
};

struct LifeState {
  bool binary = true;           // every cell is known to be 0 or 1
  uint32_t *d_pop = nullptr;    // populations of the last run, per generation
  int pop_cap = 0;
  int last_n = 0;
  int depth = 0, tile_w = 0, tile_h = 0;  // tuned or configured
};

static LifeState *life_state(Handle *h) { return (LifeState *)h->impl; }

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

// Load `count` packed words into shared memory: word i of the tile is
// row r = i / nc, column c = i % nc, global row wrap(row0 + r) and global
// word wrap(col0 + c).  One warp per word: 32 coalesced int32 loads folded
// into a word by a ballot.  8 words in flight per warp.
__device__ __forceinline__ void pack_words(const int32_t *__restrict__ cur, int n0,
                                           int n1, int wd, int row0, int col0,
                                           int nc, int count, uint32_t *dst,
                                           int warp, int nwarps, int lane) {
  for (int base = warp * 8; base < count; base += nwarps * 8) {
    int32_t v[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int i = base + j;
      v[j] = 0;
      if (i < count) {
        const int r = i / nc, c = i - (i / nc) * nc;
        int gy = (row0 + r) % n1;
        if (gy < 0) gy += n1;
        int gx = (col0 + c) % wd;
        if (gx < 0) gx += wd;
        v[j] = __ldg(cur + (size_t)gy * n0 + (size_t)gx * 32 + lane);
      }
    }
    uint32_t mine = 0;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t w = __ballot_sync(0xffffffffu, v[j] != 0);
      if (lane == j) mine = w;
    }
    if (lane < 8 && base + lane < count) dst[base + lane] = mine;
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
  pack_words(cur, n0, n1, wd, 0, 0, wd, nw, A, warp, nwarps, lane);
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
  pack_words(cur, p.n0, p.n1, p.wd, row0 - kk, col0 - 1, NC, NC * NR, A, warp,
             nwarps, lane);
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
  // write back the owned words
  const int nown = tw_own * th_own;
  for (int base = warp * 4; base < nown; base += nwarps * 4) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int i = base + j;
      if (i < nown) {
        const int r = i / tw_own, c = i - (i / tw_own) * tw_own;
        const uint32_t w = A[(r + kk) * NC + c + 1];
        next[(size_t)(row0 + r) * p.n0 + (size_t)(col0 + c) * 32 + lane] =
            (int32_t)((w >> lane) & 1u);
      }
    }
  }
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

static void life_pick_tiles(Handle *h, TbParams &p) {
  LifeState *st = life_state(h);
  p.kk = st->depth > 0 ? std::min(st->depth, 32) : 16;
  p.tw = st->tile_w > 0 ? st->tile_w : 32;
  p.th = st->tile_h > 0 ? st->tile_h : 64;
  p.tw = std::min(p.tw, p.wd);
  p.th = std::min(p.th, p.n1);
}

static size_t tb_smem_bytes(const TbParams &p) {
  return 2 * sizeof(uint32_t) * (size_t)(p.tw + 2) * (p.th + 2 * p.kk);
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
    if ((size_t)wd * n1 <= (size_t)kSmallMaxWords) {
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
      life_pick_tiles(h, p);
      const int kmax = p.kk;
      p.nt0 = (p.wd + p.tw - 1) / p.tw;
      p.nt1 = (p.n1 + p.th - 1) / p.th;
      // split the remaining generations into launches of near-equal depth
      const int rem = n - g;
      const int nl = (rem + kmax - 1) / kmax;
      const size_t smem_max = tb_smem_bytes(p);
      OM_CUDA_CHECK(cudaFuncSetAttribute(life_tb_kernel,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem_max));
      for (int l = 0; l < nl; ++l) {
        const int kk = rem / nl + (l < rem % nl ? 1 : 0);
        p.kk = kk;
        cudaEvent_t ev = prof_begin(h);
        life_tb_kernel<<<p.nt0 * p.nt1, 256, tb_smem_bytes(p), h->stream>>>(
            (const int32_t *)a.d(), (int32_t *)a.d_next(), p, st->d_pop + g);
        OM_CUDA_CHECK(cudaGetLastError());
        prof_end(h, ev, "life_tb_kernel", (double)n0 * n1 * kk);
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

static void life_array_written(Handle *h, Array *a) {
  (void)a;
  life_state(h)->binary = false;
}

static void life_free(Handle *h) {
  LifeState *st = life_state(h);
  if (st) {
    if (st->d_pop) cudaFree(st->d_pop);
    delete st;
  }
  h->impl = nullptr;
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
  const size_t smem = tb_smem_bytes(p);
  cudaError_t e = cudaFuncSetAttribute(life_tb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return e;
  life_tb_kernel<<<p.nt0 * p.nt1, 256, smem, s>>>(cur, next, p, pop);
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
  h->ops.array_written = life_array_written;
  h->ops.reserve = life_reserve;
  OM_TRY(alloc_array(h, "cell", sizeof(int32_t)));
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

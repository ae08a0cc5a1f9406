// hydro_exact.cu -- Hydro kernels built WITHOUT multiply-add contraction
// (-fmad=false for this translation unit): every operation rounds as the
// generated C++ does, so FP64 (and the exact FP32 variant) reproduce the
// oracle bit for bit.  Also: CFL minimum, plain path, initial states and
// the compensated FP64 totals.
#include <cuda_runtime.h>

#include "hydro_launch.cuh"
#include "om_internal.cuh"

namespace om {

void hydro_tile_dims(int tile, int *tx, int *ty) {
  switch (tile) {
    case kTile32x8: *tx = 32; *ty = 8; break;
    case kTile64x16: *tx = 64; *ty = 16; break;
    case kTile32x32: *tx = 32; *ty = 32; break;
    case kPersist32x32: *tx = 32; *ty = 32; break;
    case kPair32x32: *tx = 32; *ty = 32; break;
    case kPairGroups32x32: *tx = 32; *ty = 32; break;
    case kTile64x8: *tx = 64; *ty = 8; break;
    case kSweep32x8: *tx = 32; *ty = 8; break;
    case kSweep32x16: *tx = 32; *ty = 16; break;
    case kSweep64x8: *tx = 64; *ty = 8; break;
    default: *tx = 32; *ty = 16; break;
  }
}

template <class R, int TX, int TY, int NT, bool OPEN>
static cudaError_t launch_fused(const HydroStepArgs &a0, cudaStream_t s, int *grid_out) {
  HydroStepArgs a = a0;
  a.nt0 = (a.n0 + TX - 1) / TX;
  const int nt1 = (a.n1 + TY - 1) / TY;
  const size_t smem = sizeof(FusedSmem<R, TX, TY>);
  cudaError_t e = cudaFuncSetAttribute(hydro_fused_kernel<R, TX, TY, NT, OPEN>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  hydro_fused_kernel<R, TX, TY, NT, OPEN><<<a.nt0 * nt1, NT, smem, s>>>(a);
  if (grid_out) *grid_out = a.nt0 * nt1;
  return cudaGetLastError();
}

template <class R>
static cudaError_t launch_tape(const HydroStepArgs &a0, const HydroTapeOut &t, cudaStream_t s) {
  constexpr int TX = 32, TY = 16, NT = 256;
  HydroStepArgs a = a0;
  a.nt0 = (a.n0 + TX - 1) / TX;
  const int nt1 = (a.n1 + TY - 1) / TY;
  const size_t smem = sizeof(FusedSmem<R, TX, TY>);
  cudaError_t e = cudaFuncSetAttribute(hydro_fused_tape_kernel<R, TX, TY, NT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  hydro_fused_tape_kernel<R, TX, TY, NT><<<a.nt0 * nt1, NT, smem, s>>>(a, t);
  return cudaGetLastError();
}

// taped step of the FP64 and exact FP32 builds
cudaError_t hydro_fused_tape_exact(int fp64, const HydroStepArgs &a, const HydroTapeOut &t,
                                   cudaStream_t s) {
  return fp64 ? launch_tape<double>(a, t, s) : launch_tape<float>(a, t, s);
}

// a.lm > 0: open grid (margins, jet boundary condition)
cudaError_t hydro_fused_f64(const HydroStepArgs &a, int tile, cudaStream_t s, int *grid_out) {
  (void)tile;  // one shape in FP64: 32x16 (104 KB of shared memory)
  return a.lm > 0 ? launch_fused<double, 32, 16, 256, true>(a, s, grid_out)
                  : launch_fused<double, 32, 16, 256, false>(a, s, grid_out);
}

// exact FP32 variant (the fast build lives in hydro_fast.cu)
cudaError_t hydro_fused_f32_exact(const HydroStepArgs &a, cudaStream_t s, int *grid_out) {
  return a.lm > 0 ? launch_fused<float, 32, 16, 256, true>(a, s, grid_out)
                  : launch_fused<float, 32, 16, 256, false>(a, s, grid_out);
}

// CFL minimum of an open grid: margin cells (jet state) into *margin_min,
// then the interior cells and the margin minimum into sc->tsmin[slot]
cudaError_t hydro_tsmin_open(int fp64, const void *rho, const void *v0, const void *v1,
                             const void *p, int n0, int n1, int lm, double gamma,
                             HydroScalars *sc, int slot, unsigned long long *margin_min, int grid,
                             cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(margin_min, 0xFF, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  if (fp64) {
    hydro_margin_min_kernel<double><<<grid, 256, 0, s>>>(n0, n1, lm, gamma, sc, margin_min);
    hydro_tsmin_open_kernel<double><<<grid, 256, 0, s>>>(
        (const double *)rho, (const double *)v0, (const double *)v1, (const double *)p, n0, n1,
        lm, gamma, sc, slot, margin_min);
  } else {
    hydro_margin_min_kernel<float><<<grid, 256, 0, s>>>(n0, n1, lm, gamma, sc, margin_min);
    hydro_tsmin_open_kernel<float><<<grid, 256, 0, s>>>(
        (const float *)rho, (const float *)v0, (const float *)v1, (const float *)p, n0, n1, lm,
        gamma, sc, slot, margin_min);
  }
  return cudaGetLastError();
}

template <class R, int TX, int TY, int NT>
static cudaError_t launch_ensemble(const HydroStepArgs *args, const int *prefix, int count,
                                   int grid, cudaStream_t s) {
  const size_t smem = sizeof(FusedSmem<R, TX, TY>);
  cudaError_t e = cudaFuncSetAttribute(hydro_ensemble_kernel<R, TX, TY, NT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  hydro_ensemble_kernel<R, TX, TY, NT><<<grid, NT, smem, s>>>(args, prefix, count);
  return cudaGetLastError();
}

template <class R, int TX, int TY, int NT> static int occupancy_of() {
  const size_t smem = sizeof(FusedSmem<R, TX, TY>);
  cudaFuncSetAttribute(hydro_ensemble_kernel<R, TX, TY, NT>,
                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, hydro_ensemble_kernel<R, TX, TY, NT>, NT,
                                                    smem) != cudaSuccess || n < 1) {
    cudaGetLastError();
    n = 1;
  }
  return n;
}

cudaError_t hydro_ensemble_f64(const HydroStepArgs *args, const int *prefix, int count, int tile,
                               int grid, cudaStream_t s) {
  (void)tile;
  return launch_ensemble<double, 32, 16, 256>(args, prefix, count, grid, s);
}

cudaError_t hydro_ensemble_f32_exact(const HydroStepArgs *args, const int *prefix, int count,
                                     int grid, cudaStream_t s) {
  return launch_ensemble<float, 32, 16, 256>(args, prefix, count, grid, s);
}

int hydro_ensemble_occupancy_exact(int fp64) {
  return fp64 ? occupancy_of<double, 32, 16, 256>() : occupancy_of<float, 32, 16, 256>();
}

cudaError_t hydro_tsmin(int fp64, const void *rho, const void *v0, const void *v1,
                        const void *p, size_t n, double gamma, HydroScalars *sc, int slot,
                        int grid, cudaStream_t s) {
  if (fp64)
    hydro_tsmin_kernel<double><<<grid, 256, 0, s>>>((const double *)rho, (const double *)v0,
                                                    (const double *)v1, (const double *)p, n,
                                                    gamma, sc, slot);
  else
    hydro_tsmin_kernel<float><<<grid, 256, 0, s>>>((const float *)rho, (const float *)v0,
                                                   (const float *)v1, (const float *)p, n,
                                                   gamma, sc, slot);
  return cudaGetLastError();
}

cudaError_t hydro_plain_timescale(int fp64, const void *rho, const void *v0, const void *v1,
                                  const void *p, void *ts, size_t n, double gamma,
                                  const HydroScalars *sc, int grid, cudaStream_t s) {
  if (fp64)
    hydro_plain_timescale_kernel<double><<<grid, 256, 0, s>>>(
        (const double *)rho, (const double *)v0, (const double *)v1, (const double *)p,
        (double *)ts, n, gamma, sc);
  else
    hydro_plain_timescale_kernel<float><<<grid, 256, 0, s>>>(
        (const float *)rho, (const float *)v0, (const float *)v1, (const float *)p,
        (float *)ts, n, gamma, sc);
  return cudaGetLastError();
}

cudaError_t hydro_plain_reduce_min(int fp64, const void *ts, size_t n, unsigned long long *out,
                                   int grid, cudaStream_t s) {
  if (fp64)
    hydro_plain_reduce_min_kernel<double><<<grid, 256, 0, s>>>((const double *)ts, n, out);
  else
    hydro_plain_reduce_min_kernel<float><<<grid, 256, 0, s>>>((const float *)ts, n, out);
  return cudaGetLastError();
}

cudaError_t hydro_plain_step(int fp64, const void *rho, const void *v0, const void *v1,
                             const void *p, void *orho, void *ov0, void *ov1, void *op, int n0,
                             int n1, double gamma, double dtG, double dR0, double dR1, int grid,
                             cudaStream_t s) {
  if (fp64) {
    PlainView<double> V{(const double *)rho, (const double *)v0, (const double *)v1,
                        (const double *)p, n0, n1};
    hydro_plain_step_kernel<double><<<grid, 128, 0, s>>>(V, (double *)orho, (double *)ov0,
                                                         (double *)ov1, (double *)op, gamma,
                                                         dtG, dR0, dR1);
  } else {
    PlainView<float> V{(const float *)rho, (const float *)v0, (const float *)v1,
                       (const float *)p, n0, n1};
    hydro_plain_step_kernel<float><<<grid, 128, 0, s>>>(V, (float *)orho, (float *)ov0,
                                                        (float *)ov1, (float *)op, gamma,
                                                        (float)dtG, (float)dR0, (float)dR1);
  }
  return cudaGetLastError();
}

__global__ void hydro_scalar_advance_kernel(HydroScalars *sc, double dt, double *dt_hist) {
  sc->time = sc->time + dt;
  sc->dt_last = dt;
  dt_hist[0] = dt;
}

cudaError_t hydro_scalar_advance(HydroScalars *sc, double dt, double *dt_hist, cudaStream_t s) {
  hydro_scalar_advance_kernel<<<1, 1, 0, s>>>(sc, dt, dt_hist);
  return cudaGetLastError();
}

// buildInit (HydroMain.hs:79-102) over the memory array: loadIndex is the
// cell index minus the margin lm, so with the cyclic codec (lm 0) the jet
// region (x < 0) is empty, and on an open grid it lies in the left margin.
template <class R>
__global__ void hydro_init_jet_kernel(R *rho, R *v0, R *v1, R *p, int n0, int n1, int lm,
                                      double gamma, const HydroScalars *sc) {
  const int ms0 = n0 + 2 * lm;
  const size_t n = (size_t)ms0 * (n1 + 2 * lm);
  const R g = (R)gamma, dR0 = (R)sc->dR0, dR1 = (R)sc->dR1, ext1 = (R)sc->extent1;
  const R pi = (R)3.141592653589793;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / ms0), x = (int)(i - (size_t)y * ms0);
    const int iy = y - lm, ix = x - lm;
    const R cx = dR0 * (R)ix, cy = dR1 * (R)iy;
    const bool region = (cy > R(0.47) * ext1) && ((cy < R(0.53) * ext1) && (cx < R(0)));
    const R factor = R(1) + R(1e-3) * (R)sin((double)(R(6) * pi * cx));
    rho[i] = factor * g * g * (region ? R(1) : R(10));
    v0[i] = region ? R(6) : R(0);
    v1[i] = R(0);
    p[i] = factor * R(0.6);
  }
}

cudaError_t hydro_init_jet(int fp64, void *rho, void *v0, void *v1, void *p, int n0, int n1,
                           int lm, double gamma, const HydroScalars *sc, cudaStream_t s) {
  const int grid = 1024;
  if (fp64)
    hydro_init_jet_kernel<double><<<grid, 256, 0, s>>>((double *)rho, (double *)v0,
                                                       (double *)v1, (double *)p, n0, n1, lm,
                                                       gamma, sc);
  else
    hydro_init_jet_kernel<float><<<grid, 256, 0, s>>>((float *)rho, (float *)v0, (float *)v1,
                                                      (float *)p, n0, n1, lm, gamma, sc);
  return cudaGetLastError();
}

// Kelvin-Helmholtz synthetic state, computed in double, rounded once
template <class R>
__global__ void hydro_init_kh_kernel(R *rho, R *v0, R *v1, R *p, int n0, int n1,
                                     unsigned long long seed_mix) {
  const size_t n = (size_t)n0 * n1;
  const double pi = 3.141592653589793;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / n0), x = (int)(i - (size_t)y * n0);
    const double cx = (x + 0.5) / n0, cy = (y + 0.5) / n1;
    const bool band = fabs(cy - 0.5) < 0.25;
    const double u = (double)(mix64(seed_mix + (unsigned long long)i * 0x9E3779B97F4A7C15ULL) >> 11) *
                     (1.0 / 9007199254740992.0);
    rho[i] = (R)(band ? 2.0 : 1.0);
    v0[i] = (R)(band ? 0.5 : -0.5);
    v1[i] = (R)(0.01 * sin(4.0 * pi * cx) + 0.01 * (2.0 * u - 1.0));
    p[i] = (R)2.5;
  }
}

cudaError_t hydro_init_kh(int fp64, void *rho, void *v0, void *v1, void *p, int n0, int n1,
                          unsigned long long seed_mix, cudaStream_t s) {
  const int grid = 2048;
  if (fp64)
    hydro_init_kh_kernel<double><<<grid, 256, 0, s>>>((double *)rho, (double *)v0,
                                                      (double *)v1, (double *)p, n0, n1,
                                                      seed_mix);
  else
    hydro_init_kh_kernel<float><<<grid, 256, 0, s>>>((float *)rho, (float *)v0, (float *)v1,
                                                     (float *)p, n0, n1, seed_mix);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// compensated totals: each thread keeps Neumaier sums of mass, momentum x/y
// and energy over a fixed grid-stride set of cells; blocks combine them in a
// fixed tree; one block folds the block partials in index order.
// ---------------------------------------------------------------------------
struct Neu {
  double s, c;
};

__device__ __forceinline__ void neu_add(Neu &a, double x) {
  const double t = a.s + x;
  if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
  else a.c += (x - t) + a.s;
  a.s = t;
}

__device__ __forceinline__ void neu_merge(Neu &a, const Neu &b) {
  neu_add(a, b.s);
  a.c += b.c;
}

__device__ void block_merge(Neu (&v)[4], Neu (*sh)[4]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      Neu w{__shfl_down_sync(0xffffffffu, v[k].s, o), __shfl_down_sync(0xffffffffu, v[k].c, o)};
      if (lane + o < 32) neu_merge(v[k], w);
    }
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < 4; ++k) sh[warp][k] = v[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    const int nw = blockDim.x >> 5;
    for (int w = 1; w < nw; ++w)
#pragma unroll
      for (int k = 0; k < 4; ++k) neu_merge(v[k], sh[w][k]);
  }
}

template <class R>
__global__ void __launch_bounds__(256)
hydro_totals_kernel(const R *__restrict__ rho, const R *__restrict__ u, const R *__restrict__ v,
                    const R *__restrict__ p, int n0, int n1, int lm, double gamma,
                    double *partials) {
  __shared__ Neu sh[8][4];
  Neu acc[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  const size_t n = (size_t)n0 * n1;
  const int ms0 = n0 + 2 * lm;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (size_t)gridDim.x * blockDim.x) {
    // interior cell k of the memory array
    const size_t i = lm ? (size_t)((int)(k / n0) + lm) * ms0 + (int)(k % n0) + lm : k;
    const double r = rho[i], a = u[i], b = v[i], q = p[i];
    neu_add(acc[0], r);
    neu_add(acc[1], r * a);
    neu_add(acc[2], r * b);
    neu_add(acc[3], 0.5 * r * (a * a + b * b) + q / (gamma - 1.0));
  }
  block_merge(acc, sh);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      partials[blockIdx.x * 8 + 2 * k] = acc[k].s;
      partials[blockIdx.x * 8 + 2 * k + 1] = acc[k].c;
    }
}

__global__ void hydro_totals_final_kernel(const double *partials, int blocks, double *out) {
  if (threadIdx.x != 0) return;
  for (int k = 0; k < 4; ++k) {
    Neu a{0, 0};
    for (int b = 0; b < blocks; ++b) neu_merge(a, Neu{partials[b * 8 + 2 * k], partials[b * 8 + 2 * k + 1]});
    out[k] = a.s + a.c;
  }
}

cudaError_t hydro_totals(int fp64, const void *rho, const void *v0, const void *v1,
                         const void *p, int n0, int n1, int lm, double gamma, double *partials,
                         int blocks, double *out, cudaStream_t s) {
  if (fp64)
    hydro_totals_kernel<double><<<blocks, 256, 0, s>>>((const double *)rho, (const double *)v0,
                                                       (const double *)v1, (const double *)p, n0,
                                                       n1, lm, gamma, partials);
  else
    hydro_totals_kernel<float><<<blocks, 256, 0, s>>>((const float *)rho, (const float *)v0,
                                                      (const float *)v1, (const float *)p, n0,
                                                      n1, lm, gamma, partials);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  hydro_totals_final_kernel<<<1, 32, 0, s>>>(partials, blocks, out);
  return cudaGetLastError();
}

}  // namespace om

/*
 * om_oracle.h -- CPU restatement of the Orthotope Machine kernels that
 * Paraiso's generator emits for examples/Life and examples/Hydro.
 *
 * TEST INFRASTRUCTURE ONLY.  This oracle is the checker for the CUDA
 * library in paraiso_gb300/: only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it.  The product never links it.
 *
 * Storage convention (Language/Paraiso/Generator/PlanTrans.hs:136-151):
 * arrays are x-fastest, addr = (lm0+i0) + ms0*(lm1+i1), where lm is the
 * lower margin and ms the memory size of an axis.  Cyclic boundary gives
 * zero margins (Language/Paraiso/Generator/OMTrans.hs:103-116); open
 * boundary gives margins equal to the stencil radius (Life 1, Hydro 3).
 *
 * Parity pins: oracle_life_* is checked bit-exactly against the
 * reference's pre-generated examples-old/Life-exampled/dist/Life.cpp and
 * oracle_hydro_*_f32 against examples-old/Hydro-exampled/dist/Hydro.cpp
 * (open boundary, float, gamma 5/3), both compiled from the reference's
 * own sources by oracle/Makefile.
 */
#ifndef OM_ORACLE_H
#define OM_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- synthetic inputs ------------------------------------------------ */

/* Counter-based 64-bit hash of (seed, index): splitmix64 finaliser applied
 * to mix64(seed) + index * golden-ratio constant. */
uint64_t oracle_hash64(uint64_t seed, uint64_t index);

/* out[i] = (float)(lo + (hi - lo) * u_i), u_i = (hash(seed, i) >> 11) * 2^-53. */
void oracle_hash_uniform_f32(uint64_t seed, size_t n, double lo, double hi,
                             float *out);

/* Bernoulli(p) cell for interior index i = x + n0*y: alive iff
 * (hash >> 11) < floor(p * 2^53). */
void oracle_life_fill_bernoulli(int n0, int n1, int cyclic, uint64_t seed,
                                double p, int32_t *cell);

/* ---- Life (examples/Life/Generator.hs:71-115) ------------------------- */

/* Memory extent of one axis: n + 2 for open boundary, n for cyclic. */
int oracle_life_memory_size(int n, int cyclic);

/* One `proceed`: next = rule(cur), returns population = sum over the whole
 * memory array of next (int arithmetic with wraparound).  Open boundary:
 * margins of next are zero, the manifest never being written there. */
int32_t oracle_life_step(int n0, int n1, int cyclic, const int32_t *cur,
                         int32_t *next);

/* Runs `steps` generations in place, writing populations[t] (may be NULL). */
void oracle_life_run(int n0, int n1, int cyclic, int steps, int32_t *cell,
                     int32_t *populations);

/* ---- Hydro (examples/Hydro/HydroMain.hs:134-276, Hydro.hs:37-127) ----- */

typedef struct {
  int n0, n1;          /* interior size */
  int cyclic;          /* 1: periodic, margins 0; 0: open, margins 3 + jet BC */
  double gamma;        /* ratio of specific heats (kGamma) */
} oracle_hydro_shape;

int oracle_hydro_memory_size(int n, int cyclic);

/* One `proceed` in double / float.  Arrays are memory-sized.  `time` is
 * advanced by dtG = cfl * min(timescale); dtG is returned. */
double oracle_hydro_step_f64(oracle_hydro_shape s, double cfl, double dR0,
                             double dR1, double extent0, double extent1,
                             double *time, double *dens, double *vx,
                             double *vy, double *pres);
float oracle_hydro_step_f32(oracle_hydro_shape s, float cfl, float dR0,
                            float dR1, float extent0, float extent1,
                            float *time, float *dens, float *vx, float *vy,
                            float *pres);

/* The reference's `init` kernel (HydroMain.hs:79-102): jet + sin factor. */
void oracle_hydro_init_jet_f64(oracle_hydro_shape s, double dR0, double dR1,
                               double extent0, double extent1, double *dens,
                               double *vx, double *vy, double *pres);
void oracle_hydro_init_jet_f32(oracle_hydro_shape s, float dR0, float dR1,
                               float extent0, float extent1, float *dens,
                               float *vx, float *vy, float *pres);

/* Kelvin-Helmholtz synthetic state on cell centres of the unit square:
 * rho = 2 if |y-0.5|<0.25 else 1; vx = +0.5 in / -0.5 out of the band;
 * vy = 0.01 sin(4 pi x) + 0.01 (2u-1), u = (hash(seed,i)>>11) * 2^-53;
 * p = 2.5.  Computed in double (the f32 variant rounds once). */
void oracle_hydro_init_kh_f64(int n0, int n1, uint64_t seed, double *dens,
                              double *vx, double *vy, double *pres);
void oracle_hydro_init_kh_f32(int n0, int n1, uint64_t seed, float *dens,
                              float *vx, float *vy, float *pres);

/* Compensated (Neumaier) sums of mass, x/y momentum and total energy over
 * the interior, in double.  out[4]. */
void oracle_hydro_totals_f64(oracle_hydro_shape s, const double *dens,
                             const double *vx, const double *vy,
                             const double *pres, double *out);
void oracle_hydro_totals_f32(oracle_hydro_shape s, const float *dens,
                             const float *vx, const float *vy,
                             const float *pres, double *out);

/* Tangent-linear (forward-mode) Hydro step in double: propagates the
 * direction (d*) through one proceed including the dependence of dt on the
 * state (through the arg-min cell).  Primal arrays are advanced too. */
double oracle_hydro_step_tl_f64(oracle_hydro_shape s, double cfl, double dR0,
                                double dR1, double *time, double *dens,
                                double *vx, double *vy, double *pres,
                                double *d_dens, double *d_vx, double *d_vy,
                                double *d_pres);

/* Floating-point operations of one Hydro step of the n0 x n1 periodic
 * Kelvin-Helmholtz start, counted on this restatement (each face's flux once,
 * only the HLLC branch taken): out[6] = {add/sub, mul, div, sqrt, compare,
 * abs/neg} summed over the step. */
void oracle_hydro_count_ops(int n0, int n1, uint64_t seed, double gamma, double cfl,
                            long long *out);

/* Number of OpenMP threads the oracle uses (1 when built without OpenMP). */
int oracle_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif

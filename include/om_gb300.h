/*
 * om_gb300.h -- C ABI of the GB300 (sm_103a) Orthotope Machine runtime.
 *
 * Paraiso's generator (Language/Paraiso/Generator/PlanTrans.hs) prints one
 * C++ class per Orthotope Machine.  Its members -- constructor, size and
 * margin accessors, scalar/array accessors, named kernels such as
 * init/proceed -- are what drivers such as examples/Life/main.cpp and
 * examples/Hydro/main-kh.cpp call.  This header exposes the same members
 * as plain C functions over an opaque handle, so the header-only shims
 * include/Life.hpp and include/Hydro.hpp rebuild the generated class on
 * top of it, and any FFI (ctypes, cgo, JNI) can bind it.
 *
 * Conventions
 *  - Every entry point returns om_status; OM_OK is 0.  On failure,
 *    om_last_error() returns a thread-local description.  (The generated
 *    class has no runtime error reporting at all.)
 *  - Arrays are stored x-fastest with margins:
 *      addr = (lower_margin_0 + i0) + memory_size_0 * (lower_margin_1 + i1)
 *    (PlanTrans.hs:136-151).  Cyclic boundary has zero margins
 *    (Language/Paraiso/Generator/OMTrans.hs:103-116).
 *  - Host/device mirror semantics follow the generated CUDA container
 *    (PlanTrans.hs:724-728): om_array_host marks the host copy newer and
 *    the next kernel uploads it; om_array_host_const only refreshes it.
 *  - A handle is not thread-safe; use one handle per host thread, as with
 *    the generated class.  All work is queued on the handle's stream and
 *    every om_run returns with that stream synchronised.
 */
#ifndef OM_GB300_H
#define OM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  OM_OK = 0,
  OM_ERR_ARG = 1,          /* bad argument, unknown name, size out of range */
  OM_ERR_CUDA = 2,         /* CUDA runtime error (text in om_last_error) */
  OM_ERR_UNSUPPORTED = 3,  /* configuration not implemented */
  OM_ERR_NOMEM = 4,        /* device or pinned host allocation failed */
  OM_ERR_NONFINITE = 5,    /* a NaN/Inf was detected in a reduction */
  OM_ERR_TIMEOUT = 6,      /* a bounded device-side wait gave up */
  OM_ERR_STATE = 7         /* call not valid in the handle's current state */
} om_status;

typedef enum { OM_KIND_LIFE = 1, OM_KIND_HYDRO = 2, OM_KIND_GRAPH = 3 } om_kind;
typedef enum { OM_BOUNDARY_CYCLIC = 0, OM_BOUNDARY_OPEN = 1 } om_boundary;
typedef enum { OM_SCALAR_INT = 0, OM_SCALAR_DOUBLE = 1 } om_scalar_type;

typedef struct om_handle_s *om_handle;

/* Runtime counterpart of Native.Setup (Language/Paraiso/Generator/Native.hs:16-24):
 * boundary per OM, plus the knobs the GB300 kernels expose to the tuner. */
typedef struct {
  int boundary;     /* om_boundary; applies to every axis */
  int precision;    /* Hydro: 32 = FP32 bulk with FP64 dt and totals; 64 = FP64 */
  double gamma;     /* Hydro: ratio of specific heats (kGamma, examples/Hydro/Hydro.hs:53-54) */
  int device;       /* CUDA device ordinal */
  int depth;        /* Life: generations per temporally blocked launch (0 = tuned) */
  int tile_x;       /* Life: tile width in 32-cell words; Hydro: tile width in cells (0 = tuned) */
  int tile_y;       /* tile height in cells (0 = tuned; Hydro FP32: 0 = the persistent
                       32 x 32 kernel on grids whose sides are multiples of 32 and
                       at least 64 (else the 32 x 32 tile kernel): with tile_x 0
                       paired, as one CTA per SM of two groups half a tile apart
                       when every group gets at least 16 tiles, else two CTAs per
                       SM; with tile_x 16 paired, two CTAs per SM; with tile_x 32
                       one wall per thread.  8, 16 and 32 with tile_x 0 or 32, 8
                       and 16 with tile_x 64 are tile kernels; a negative -k
                       selects the column sweep of k rows per chunk, 8 or 16) */
  int use_graph;    /* capture om_run_n in a CUDA graph (default 1) */
  int variant;      /* 0 = fastest path.  Life 1: integer one-cell-per-thread kernel only.
                       Hydro 1: plain unfused FP64-structured grid-stride kernels */
  int life_io;      /* Life cell I/O of the packed kernels: 0 = 128-bit, 1 = 32-bit */
  int life_kernel;  /* Life packed kernel: k >= 1 = warp-specialised persistent
                       kernel, variant k-1 (variants 4-10 and 13-15 take their rows
                       by TMA and need rows of at least 1024 cells; in 14 and 15
                       each consumer warp synchronises with its two neighbours
                       only); 0 = automatic:
                       with tile_y 0, that kernel on grids of at least 1.5 of its
                       tiles per SM, else register-resident blocks */
  int grid_limit;   /* persistent kernels (Life warp-specialised, the persistent
                       Hydro FP32 step, Hydro ensembles): at most this many
                       CTAs (0 = as many as the GPU keeps resident) */
  int reserved[4];
} om_config;

/* Fill `cfg` with defaults: cyclic, FP32, gamma 5/3, device 0, tuned tiles. */
void om_config_default(om_config *cfg);

/* Text of the last error raised on this host thread ("" if none). */
const char *om_last_error(void);

/* Library version string. */
const char *om_version(void);

/* ---- construction ----------------------------------------------------- */

/* Replaces the generated class constructor (PlanTrans.hs:75-86), with the
 * mesh size (Native.localSize) given at run time.  kind: om_kind; ndim: 2;
 * sizes[ndim]: interior extent per axis.  Allocates every array with
 * om_memory_size elements, zero-filled, as the generated constructor does. */
om_status om_create(int kind, int ndim, const int *sizes, const om_config *cfg,
                    om_handle *out);

/* Releases the handle and all its device and host memory. */
om_status om_destroy(om_handle h);

/* ---- sizes (PlanTrans.hs:167-215) -------------------------------------
 * axis = -1 gives the product over axes (om_size / om_memory_size). */
om_status om_size(om_handle h, int axis, int *out);
om_status om_memory_size(om_handle h, int axis, int *out);
om_status om_lower_margin(om_handle h, int axis, int *out);
om_status om_upper_margin(om_handle h, int axis, int *out);

/* ---- kernels (PlanTrans.hs:225-277) ------------------------------------ */

/* Kernel index by name ("init", "proceed", ...). */
om_status om_kernel_id(om_handle h, const char *name, int *id);
/* Runs one kernel: `void init()` / `void proceed()` of the generated class. */
om_status om_run(om_handle h, int kernel_id);
/* Runs a kernel n times back to back (a driver's step loop), captured in a
 * CUDA graph when cfg.use_graph is set.  Scalars are synced once at the end. */
om_status om_run_n(om_handle h, int kernel_id, int n);

/* ---- static variable accessors (PlanTrans.hs:117-157) ------------------ */

/* Host pointer to a Scalar static (`T& name()`); valid for the handle's
 * lifetime.  Writes take effect at the next om_run; om_run refreshes it. */
om_status om_scalar_ptr(om_handle h, const char *name, void **ptr, int *type);

/* Host mirror of an Array static (`container<T>& name()`, `T& name(i0,i1)`),
 * memory-sized.  Downloads if the device copy is newer, then marks the host
 * copy newer so the next kernel uploads it (thrust_vector::operator[]). */
om_status om_array_host(om_handle h, const char *name, void **ptr,
                        size_t *count, int *elem_size);
/* Same, read-only: refreshes the host copy without marking it newer. */
om_status om_array_host_const(om_handle h, const char *name, const void **ptr,
                              size_t *count, int *elem_size);
/* Device pointer of an Array static (thrust_vector::raw()): uploads if the
 * host copy is newer, then marks the device copy newer.  Valid until the
 * next kernel (statics are double-buffered and swap on every step). */
om_status om_array_device(om_handle h, const char *name, void **dptr);
/* Copy an array out of / into caller memory (host or device pointer;
 * cudaMemcpyDefault), memory-sized. */
om_status om_array_read(om_handle h, const char *name, void *dst, size_t bytes);
om_status om_array_write(om_handle h, const char *name, const void *src, size_t bytes);

/* ---- synthetic inputs and extra results (no counterpart in the generated
 * class: benchmark inputs and multi-step reduce results) ---------------- */

/* Life: every interior cell i = x + n0*y alive iff
 * (splitmix-style hash(seed, i) >> 11) < floor(p * 2^53); margins 0. */
om_status om_life_fill_random(om_handle h, uint64_t seed, double p);
/* Life: populations after each generation of the last om_run / om_run_n
 * (the `reduce Sum` of examples/Life/Generator.hs:110).  Copies min(n, kept). */
om_status om_life_population_history(om_handle h, int32_t *out, int n, int *written);

/* Hydro: Kelvin-Helmholtz state on cell centres of the unit square (periodic):
 * rho 2 in |y-0.5|<0.25 else 1, vx +0.5/-0.5, vy = 0.01 sin(4 pi x) +
 * 0.01 (2u-1), u = (hash(seed,i) >> 11) 2^-53, p 2.5; sets extent 1,
 * dR = 1/n, time 0. */
om_status om_hydro_init_kh(om_handle h, uint64_t seed);
/* Hydro: compensated FP64 sums over the interior of mass, x momentum,
 * y momentum and total energy (out[4]); OM_ERR_NONFINITE if any is not finite. */
om_status om_hydro_totals(om_handle h, double *out);
/* Hydro: dt of each step of the last om_run / om_run_n. */
om_status om_hydro_dt_history(om_handle h, double *out, int n, int *written);

/* ---- adjoint (no counterpart in the reference) -------------------------- */

/* One reverse-mode step at the handle's current state: cot_next[4] (device
 * arrays, memory-sized: cotangent of density, velocity0, velocity1, pressure
 * after one proceed) -> cot_prev[4] (cotangent of the current state),
 * through both stages, MUSCL-minmod, HLLC, the clamps and the step's CFL dt
 * (routed to the arg-min cell of the timescale). */
om_status om_hydro_vjp(om_handle h, void *const *cot_next, void *const *cot_prev);
/* Checkpointed forward/backward pair.  om_hydro_forward runs `steps` proceed
 * steps from the current state and keeps the state every `checkpoint_every`
 * steps (0: ceil(sqrt(steps))) in a tape; the handle ends at the final
 * state.  om_hydro_backward maps dL/d(final state) (cot_final[4]: density,
 * velocity0, velocity1, pressure; host or device arrays of om_memory_size
 * elements) to dL/d(start state) in grad[4] (host or device), recomputing
 * each segment from its checkpoint; the handle is left at the final state
 * and the tape serves any number of cotangents until om_hydro_tape_free. */
typedef struct om_hydro_tape_s *om_hydro_tape;
om_status om_hydro_forward(om_handle h, int steps, int checkpoint_every, om_hydro_tape *tape);
om_status om_hydro_backward(om_handle h, om_hydro_tape tape, const void *const *cot_final,
                            void *const *grad);
om_status om_hydro_tape_free(om_hydro_tape tape);
/* Gradient of loss = mean((density_T - target)^2) over `steps` proceed
 * steps from the current state, w.r.t. that state (grad[4]: host or device
 * arrays), with checkpoints every `checkpoint_every` steps (0: sqrt(steps)).
 * The handle ends at the final state; *loss receives the loss. */
om_status om_hydro_adjoint_run(om_handle h, int steps, const void *target,
                               int checkpoint_every, double *loss, void *const *grad);
/* Device time (ms, mean of reps) of one adjoint step at the current state:
 * the reverse sweep from the step's tape.  The tape (stage-1 state and both
 * stages' flux differences) is written by the forward step itself when the
 * backward pass recomputes a segment from its checkpoint; its cost is
 * om_hydro_time_tape's. */
om_status om_hydro_time_vjp(om_handle h, int reps, float *ms);
/* Device time (ms, mean of reps) of one taped forward step at the current
 * state; the handle does not move. */
om_status om_hydro_time_tape(om_handle h, int reps, float *ms);

/* ---- measurement ------------------------------------------------------- */

/* Runs a kernel n times inside CUDA events on the handle's stream and
 * returns the elapsed device time in milliseconds. */
om_status om_time_run(om_handle h, int kernel_id, int n, float *ms);
/* Number of kernel launches issued by the last om_run / om_run_n / om_time_run. */
om_status om_last_launch_count(om_handle h, int *launches);
/* Per-launch device timing: while enabled, every kernel launch is bracketed
 * by CUDA events on the handle's stream (runs then skip graph capture).
 * Disabling clears the totals. */
om_status om_profile_enable(om_handle h, int enable);
/* Totals for one kernel (by its __global__ name, e.g. "life_tb_kernel"):
 * launches, summed device milliseconds and summed work units (cell-updates). */
om_status om_profile_query(om_handle h, const char *kernel, long *launches,
                           double *total_ms, double *total_units);

/* ---- autotuning (replaces the reference's genetic-algorithm tuning loop,
 * Language/Paraiso/Tuning/Genetic.hs) ------------------------------------ */

/* Times every candidate of a small grid of launch knobs on a mesh of this
 * size and returns the fastest configuration (and its cell-updates/s).
 * Life: kernel family, temporal depth, block rows; Hydro: fused tile shape.
 * `base` fixes everything else (boundary, precision, gamma, device).
 * Results are cached per (kind, size, precision, device) in the process. */
om_status om_autotune(int kind, int ndim, const int *sizes, const om_config *base,
                      om_config *best, double *best_rate);

/* ---- batched Hydro ensembles (no counterpart in the reference) ---------- */

typedef struct om_ensemble_s *om_ensemble;

/* count independent periodic Hydro grids, sizes[2k], sizes[2k+1] = n0, n1 of
 * instance k (uneven sizes allowed).  cfg: precision 32 (variant 0 fast or
 * 2 exact) or 64, gamma, tile_x 64 / tile_y 8 pick the FP32 tile shape.
 * Every instance starts with cfl 0.4, extent 1, dR = 1/n, time 0. */
om_status om_ensemble_create(int count, const int *sizes, const om_config *cfg,
                             om_ensemble *out);
om_status om_ensemble_destroy(om_ensemble e);
/* count, total interior cells, persistent grid size, tile work items */
om_status om_ensemble_info(om_ensemble e, int *count, long long *total_cells, int *grid,
                           int *work_items);
/* Kelvin-Helmholtz state of om_hydro_init_kh in every instance, seed base+k. */
om_status om_ensemble_init_kh(om_ensemble e, uint64_t base_seed);
/* n steps: one persistent launch per step over every (instance, tile), each
 * instance with its own CFL dt and time; replayed from a CUDA graph. */
om_status om_ensemble_step(om_ensemble e, int n);
/* n steps timed with CUDA events on the ensemble's stream (milliseconds). */
om_status om_ensemble_time_step(om_ensemble e, int n, float *ms);
/* Copy field ("density", "velocity0", "velocity1", "pressure") of instance k
 * (n0*n1 elements, host or device memory). */
om_status om_ensemble_read(om_ensemble e, int k, const char *field, void *dst, size_t bytes);
om_status om_ensemble_write(om_ensemble e, int k, const char *field, const void *src,
                            size_t bytes);
/* Scalars of instance k: "time", "cfl", "dR0", "dR1", "dt" (last step). */
om_status om_ensemble_scalar(om_ensemble e, int k, const char *name, double *value);
om_status om_ensemble_set_scalar(om_ensemble e, int k, const char *name, double value);
/* Compensated FP64 totals (mass, momentum x/y, energy) of instance k. */
om_status om_ensemble_totals(om_ensemble e, int k, double *out);
om_status om_ensemble_last_launch_count(om_ensemble e, int *launches);
/* Autotune the ensemble's tile shape for these instance sizes. */
om_status om_autotune_ensemble(int count, const int *sizes, const om_config *base,
                               om_config *best, double *best_rate);

/* ---- checkpoints and snapshots (no counterpart: the generated class has
 * no I/O; its drivers print through the accessors) ------------------------ */

/* Binary checkpoint of every static (arrays, margins included, and
 * scalars) with a header describing the handle's layout. */
om_status om_save(om_handle h, const char *path);
/* Restore a checkpoint into a handle of the same kind, mesh, margins and
 * statics (OM_ERR_ARG and a reason otherwise). */
om_status om_load(om_handle h, const char *path);
/* Hydro: the text snapshot of examples/Hydro/main-kh.cpp:17-31, one line
 * "x y density velocity0 velocity1 pressure" per interior cell (cell
 * centres dR (i + 0.5)), a blank line after each row. */
om_status om_hydro_write_snapshot(om_handle h, const char *path);

/* ---- general OM graphs ---------------------------------------------------
 * The generator's input (Language/Paraiso/OM/Graph.hs:113-123: Load, Store,
 * Shift, Imm, Arith, Reduce, Broadcast, LoadIndex, LoadSize) as text, one
 * node per line, compiled at run time into CUDA kernels for this GPU:
 *
 *   om NAME NDIM N0 [N1] cyclic|open
 *   static NAME array|scalar int|float|double|bool
 *   kernel NAME
 *   ID load REALM TYPE STATIC         ID imm REALM TYPE LITERAL
 *   ID shift array TYPE NODE V0 [V1]  ID loadindex array int AXIS
 *   ID loadsize scalar int AXIS       ID reduce scalar TYPE sum|min|max NODE
 *   ID broadcast array TYPE NODE      ID OP REALM TYPE NODE...  (add sub mul
 *     div mod neg inv not and or eq ne lt le gt ge select max min abs signum
 *     sqrt exp log sin cos tan asin acos atan atan2 pow cast)
 *   store STATIC NODE
 *   manifest NODE     (Alloc.Manifest: the array value is computed once per
 *                      run into a temporary array that later passes read,
 *                      instead of being recomputed where it is used)
 *   end
 *
 * (paraiso_gb300/omgraph.py writes it from Builder-style Python.)  The
 * handle then works as any other: kernels by name (om_kernel_id, om_run),
 * statics through om_scalar_ptr / om_array_* with the margins an open mesh
 * needs.  Scalar types: 0 int (and bool), 1 double, 2 float. */
om_status om_create_graph(const char *text, const om_config *cfg, om_handle *out);
/* The CUDA source generated for a graph handle (owned by the handle). */
om_status om_graph_source(om_handle h, const char **source);
/* Parse, plan, generate and compile a graph for sm_<major><minor>a without a
 * device (no handle); *source, if given, receives the generated CUDA source
 * (valid until the next call on this thread). */
om_status om_graph_check(const char *text, int major, int minor, const char **source);

/* ---- caller-owned buffers, no allocation -------------------------------- */

/* No counterpart in the reference.  Checks the bounded wait of the TMA
 * kernels on `device`: a one-block kernel arms an mbarrier for bytes that no
 * copy delivers (none is issued), waits with a short bound (about 4 ms) and
 * must report the time-out through its error word.  OM_OK when it did. */
om_status om_selftest_wait_bound(int device);

/* Largest `generations` one om_life_proceed_noalloc call accepts. */
#define OM_LIFE_NOALLOC_MAX_GENERATIONS 32

/* No counterpart in the reference.  Advances a cyclic Life grid by
 * `generations` (1..OM_LIFE_NOALLOC_MAX_GENERATIONS) without allocating any
 * memory, for callers that cannot call cudaMalloc (under a host framework
 * whose allocator owns all device memory, in a real-time loop that must not
 * block on the allocator).  cells_in / cells_out: distinct device buffers of
 * n0*n1 int32 on the current device, n0 a multiple of 32 in [32, 2^20], n1 in
 * [1, 2^20], n0*n1 at most 2^31 - 1 (the populations are int32), every cell 0
 * or 1 (otherwise OM_ERR_ARG and cells_out is unspecified).  populations:
 * caller memory (host or device) receiving the population after each
 * generation.  stream: a cudaStream_t, or NULL for the default stream; the
 * call returns with it synchronised.  Scratch is a fixed device array shared
 * by all calls: the first call on each device looks up its address (make
 * that first call before any stream capture), and calls that overlap on the
 * GPU race. */
om_status om_life_proceed_noalloc(const int32_t *cells_in, int32_t *cells_out, int n0,
                                  int n1, int generations, int32_t *populations,
                                  void *stream);

#ifdef __cplusplus
}
#endif
#endif

/*
 * shll.h -- C-ABI of libshll_gb300.so, the GB300 (sm_103a) SHLL finite-volume Euler solver.
 *
 * The library replaces the hot path of the reference project archembaud/shll-sve-cfd: the
 * split-flux evaluation, interface flux sum and conservative update inside the explicit time
 * loop of base-c/base_shll.c (1D, first order), base-c/2nd_order_base_shll.c (second order;
 * its x sweep is the 1D second-order scheme) and base-c/base_shll_2d.c (2D, first order).
 *
 * The reference has no library API: each solver is a program whose stages are global-state
 * functions  void Allocate_and_Init_Memory(void), Compute_U_from_P, Compute_P_from_U,
 * Compute_F_from_P, Update_U_from_F, Save_Results, Free_Memory  driven by main().  This header
 * keeps those stages as calls on a context (so several problems can live in one process) and
 * also exports the reference's own void names on a default context (shll_ref_*), so that a
 * reference-style main() links unchanged.
 *
 * Conventions: every call that can fail returns int (SHLL_OK = 0, negative = error) and
 * shll_last_error() describes the last failure of that context.  All pointers in the
 * signatures are HOST pointers; device memory is owned by the context.  2D fields use the
 * reference's layout, cell index = i*ny + j (y contiguous), i.e. base-c/base_shll_2d.c:94-101.
 */
#ifndef SHLL_GB300_H
#define SHLL_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SHLL_OK 0
#define SHLL_ERR_ARG (-1)         /* invalid argument or parameter */
#define SHLL_ERR_CUDA (-2)        /* CUDA runtime error (message in shll_last_error) */
#define SHLL_ERR_STATE (-3)       /* call out of order (e.g. stage call before init) */
#define SHLL_ERR_NOMEM (-4)       /* device or host allocation failed */
#define SHLL_ERR_NUMERIC (-5)     /* non-positive density/temperature or NaN detected */
#define SHLL_ERR_TIMEOUT (-6)     /* a bounded device-side wait expired */
#define SHLL_ERR_UNSUPPORTED (-7) /* combination not implemented (e.g. stage calls in mixed mode) */

/* ---- arithmetic of the time loop ---- */
enum shll_precision {
    /* FP64 throughout, as the reference with float replaced by double.  Multiply-adds may be
     * fused (the only licensed difference from the CPU reference). */
    SHLL_PREC_F64 = 0,
    /* FP64 throughout with no fused multiply-add: bit-identical to the FP64 reference build. */
    SHLL_PREC_F64_EXACT = 1,
    /* The reference as published: float arrays with the double promotions its double
     * literals and sqrt() cause, no fused multiply-add; bit-identical to base-c built by gcc
     * on x86-64. */
    SHLL_PREC_F32_EXACT = 2,
    /* Split fluxes in FP32 (perturbation form about per-segment FP64 anchor states), state in
     * FP64; per-step increments are summed in compensated FP32 for fold_steps steps and then
     * added to the FP64 state.  fold_steps = 1 adds every step into FP64. */
    SHLL_PREC_MIXED_F64 = 3,
    /* Split fluxes in FP32 as above; the state is an FP32 value plus its FP32 compensation
     * (Kahan / float-float), with no FP64 arithmetic per cell. */
    SHLL_PREC_MIXED_KAHAN = 4
};

/* ---- initial conditions ---- */
enum shll_ic_kind {
    SHLL_IC_SOD = 0,         /* 1D: left state for i < x_d*nx, right state otherwise
                                (base-c/base_shll.c:53-60 with x_d = 0.5) */
    SHLL_IC_REF_BOX2D = 1,   /* 2D: base-c/base_shll_2d.c:92-103 (rho 1 inside (0.2,0.8)^2, 10 outside) */
    SHLL_IC_CIRCLE2D = 2,    /* 2D: "in" state strictly inside a circle of cell centres, else "out" */
    SHLL_IC_FOUR_SHOCK2D = 3,/* 2D: base-c/2nd_order_base_shll.c:133-149 */
    SHLL_IC_USER = 4,        /* primitives supplied later with shll_set_primitives() */
    SHLL_IC_QUADRANTS2D = 5  /* 2D: base-omp/2nd_order_base_shll.c:147-172 ("Configuration 6") */
};

typedef struct shll_ic {
    int kind;                      /* enum shll_ic_kind */
    double x_d;                    /* SOD: diaphragm position as a fraction of the tube */
    double rho_l, u_l, T_l;        /* SOD: left state; CIRCLE2D: inside state (u ignored) */
    double rho_r, u_r, T_r;        /* SOD: right state; CIRCLE2D: outside state (u ignored) */
    double cx, cy, radius;         /* CIRCLE2D: centre and radius in domain units */
} shll_ic;

typedef struct shll_params {
    int dim;           /* 1 or 2 */
    int order;         /* 1: first order, reflective walls (base_shll.c, base_shll_2d.c)
                          2: second order, minmod slopes of the split fluxes, outflow walls
                             (2nd_order_base_shll.c) */
    int nx, ny;        /* cells (ny ignored in 1D); nx, ny >= 2 */
    double gamma, R;   /* ratio of specific heats, gas constant (reference: 1.4, 1.0) */
    double cfl;        /* kinetic CFL: DT = (cfl/(R+1)) * DX as base_shll.c:83 (reference 0.25) */
    double lx, ly;     /* domain lengths (reference 1.0) */
    double t_end;      /* run while time < t_end ... */
    long n_steps;      /* ... unless n_steps > 0: then exactly n_steps steps */
    int precision;     /* enum shll_precision */
    int limiter;       /* order 2 only: 0 minmod (base-c), 1 MC limiter (base-omp/2nd_order_base_shll.c:316-325) */
    double mc_alpha;   /* MC limiter alpha (base-omp: 1.25) */
    int fold_steps;    /* MIXED_F64: steps between FP64 folds; 0 = library default */
    int clock_f32;     /* 1: time accumulates in float as the published reference (default for
                          F32_EXACT); 0: double, as the FP64 reference build */
    shll_ic ic;
} shll_params;

typedef struct shll_ctx shll_ctx;

/* Fills p with the reference's defaults for (dim, order): gamma 1.4, R 1, CFL 0.25, L = 1,
 * Sod (1D), reference box (2D first order) or four-shock (2D second order) initial data,
 * t_end 0.2 / 0.1 / 0.8 (base_shll.c:26, base_shll_2d.c:35, 2nd_order_base_shll.c:43),
 * nx = ny = 256, precision F64. */
void shll_params_default(shll_params* p, int dim, int order);

/* Step count of the reference time loop for these parameters: time += DT (in float when
 * clock_f32, else double) while time < t_end; or n_steps when > 0. */
long shll_steps_for(const shll_params* p);

/* Creates a context on the current CUDA device (allocates its device state). */
int shll_create(const shll_params* p, shll_ctx** out);
void shll_destroy(shll_ctx* ctx);
const char* shll_last_error(const shll_ctx* ctx);
const char* shll_status_string(int status);
/* Binds the context's work to a cudaStream_t (NULL = the context's own stream). */
int shll_set_stream(shll_ctx* ctx, void* cuda_stream);

/* ---- the reference's stages (base-c/base_shll.c:28-177) ---- */
/* Allocate_and_Init_Memory (:28-61): primitives from p->ic on the device.  Also computes U
 * from P and P from U (main() :204-205), so the context is ready to step. */
int shll_init_state(shll_ctx* ctx);
/* The initial primitives of p's initial-condition descriptor (host arrays of nx*ny doubles; v
 * ignored in 1D): the values shll_init_state loads (no counterpart in the reference, whose
 * Allocate_and_Init_Memory writes them into its globals). */
int shll_initial_primitives(const shll_params* p, double* rho, double* u, double* v, double* T);
/* Replaces the primitives (host arrays of nx*ny doubles; v ignored in 1D) and recomputes U and
 * P as shll_init_state does; SHLL_ERR_ARG if a density or temperature is not positive.  In the
 * mixed modes the arrays are copied as given (at full link speed from pinned host memory) and
 * converted on the device; shll_get_primitives likewise converts on the device. */
int shll_set_primitives(shll_ctx* ctx, const double* rho, const double* u, const double* v,
                        const double* T);
int shll_compute_U_from_P(shll_ctx* ctx);   /* base_shll.c:74-85 */
int shll_compute_P_from_U(shll_ctx* ctx);   /* base_shll.c:161-177 */
int shll_compute_F_from_P(shll_ctx* ctx);   /* base_shll.c:130-159 (split fluxes) */
int shll_update_U_from_F(shll_ctx* ctx);    /* base_shll.c:87-128 (stencil + update) */

/* ---- fused time stepping ---- */
/* Advances n steps (F -> update -> P per step, fused on the device). */
int shll_step(shll_ctx* ctx, long n);
/* The time loop of main() (base_shll.c:207-218): runs the remaining steps of
 * shll_steps_for(p).  *steps_taken (may be NULL) receives the total steps of the context. */
int shll_run(shll_ctx* ctx, long* steps_taken);
long shll_steps_taken(const shll_ctx* ctx);

/* ---- checkpoint / resume on the device ----
 * The reference keeps no checkpoint (results.dat is its only output).  shll_checkpoint copies
 * the state and the step counter into device memory owned by the context; shll_restore puts
 * them back, so a run can be repeated from the same state or split at any step. */
int shll_checkpoint(shll_ctx* ctx);
int shll_restore(shll_ctx* ctx);
/* Number of CUDA kernels this library has launched in the process so far. */
long shll_kernel_launches(void);

/* ---- results (host copies) ---- */
int shll_get_primitives(shll_ctx* ctx, double* rho, double* u, double* v, double* T);
/* conserved planes rho, rho*u, [rho*v,] E, each nx*ny doubles, written contiguously */
int shll_get_conserved(shll_ctx* ctx, double* planes);
/* split-flux planes of the last shll_compute_F_from_P (fp, fm; hp, hm in 2D may be NULL) */
int shll_get_fluxes(shll_ctx* ctx, double* fp, double* fm, double* hp, double* hm);
/* FP64 sums over all cells of rho, rho*u, [rho*v,] E (device reduction); out has 3 or 4 */
int shll_totals(shll_ctx* ctx, double* out);
/* Save_Results (base_shll.c:180-192, base_shll_2d.c:322-340): text file of
 * x [y] rho u [v] T per cell, "%e" tab-separated, x = (i+0.5)*DX in the reference's float */
int shll_save_results(shll_ctx* ctx, const char* path);

/* ---- batches of independent tubes / domains ---- */
typedef struct shll_batch shll_batch;
/* items: count parameter sets (all dim 1, or all dim 2, any sizes/orders/initial data), all
 * with one precision: SHLL_PREC_F64 or SHLL_PREC_F64_EXACT (the plain FP64 arithmetic, with or
 * without fused multiply-add, one launch per time step over every item) or a MIXED mode (the
 * sweep engine in 1D; in 2D one step launch per time step over every tile of every domain, first
 * or second order, with one order and, for second order, one limiter for all items of the batch:
 * SHLL_ERR_ARG otherwise).  SHLL_PREC_F32_EXACT batches: SHLL_ERR_UNSUPPORTED. */
int shll_batch_create(const shll_params* items, int count, shll_batch** out);
/* Runs every item to its own end (its own DT and step count). */
int shll_batch_run(shll_batch* b);
/* Runs the batch's work on a cudaStream_t (NULL = its own stream). */
int shll_batch_set_stream(shll_batch* b, void* cuda_stream);
int shll_batch_get_primitives(shll_batch* b, int item, double* rho, double* u, double* v,
                              double* T);
/* Replaces item `item`'s state with host primitive planes (v only in 2D), as shll_set_primitives
 * does for a context: copied as given (at full link speed from pinned host memory) and converted
 * on the device; SHLL_ERR_ARG with the state unchanged if a density or temperature is not
 * positive. Mixed-precision batches (SHLL_ERR_UNSUPPORTED for FP64 batches). */
int shll_batch_set_primitives(shll_batch* b, int item, const double* rho, const double* u,
                              const double* v, const double* T);
/* Every item at once (mixed-precision batches): `prim` holds, item after item in batch order,
 * each item's planes rho, u, [v,] T of nx*ny doubles.  One host<->device copy each way and one
 * synchronisation; set checks every item before changing any state (SHLL_ERR_ARG names the first
 * item and cell with a non-positive density or temperature). */
int shll_batch_set_all_primitives(shll_batch* b, const double* prim);
int shll_batch_get_all_primitives(shll_batch* b, double* prim);
int shll_batch_totals(shll_batch* b, int item, double* out);
/* SHLL_OK, or SHLL_ERR_NUMERIC if this item reached a non-positive or NaN density/energy (the
 * other items are unaffected; shll_batch_run returns SHLL_ERR_NUMERIC if any item did). */
int shll_batch_item_status(shll_batch* b, int item);
long shll_batch_cell_updates(const shll_batch* b);
const char* shll_batch_last_error(const shll_batch* b);
void shll_batch_destroy(shll_batch* b);
/* Autotuner of the mixed-precision 1D engine (no counterpart in the reference): times short runs
 * of the batch (trial_steps steps each; 0 picks a length) for candidate sweep lengths (the
 * temporal-blocking depth: 8, 16, 32 steps, which sets each chunk's owned and halo cells) and fold
 * windows (1 to 8 sweeps) and chunk sizes (the largest window, or half of it: more blocks per SM),
 * first one choice for all tubes, then per size class (order, limiter,
 * floor(log2 cells)) for the classes holding a tenth of the work or more.  The state is restored
 * afterwards (the batch's or context's device checkpoint is replaced by the current state); the
 * choices are kept process-wide and applied to later batches and contexts whose items leave
 * fold_steps at 0.  shll_batch_tuning reports an item's sweep length and fold
 * interval (steps) and its owned cells per chunk (any pointer may be NULL). */
int shll_batch_autotune(shll_batch* b, int trial_steps);
int shll_batch_tuning(shll_batch* b, int item, int* sweep_steps, int* fold_steps, int* chunk_cells);

/* Device-side checkpoint and restore of a mixed-precision batch, 1D or 2D (no counterpart in the
 * reference); restore also clears the breakdown flags raised after the checkpoint.
 * SHLL_ERR_UNSUPPORTED for FP64 batches. */
int shll_batch_checkpoint(shll_batch* b);
int shll_batch_restore(shll_batch* b);

/* ---- advancing a tube without allocating device memory ----
 * No counterpart in the reference (which has no GPU path).  For callers that cannot call
 * cudaMalloc when they need to step: a process whose device allocator is reserved or capped by
 * its host framework, a time-critical loop that must not wait on the allocator, or a host that
 * hands the library device buffers it manages itself.  d_cons is the caller's device buffer of
 * the tube's conserved variables (planes rho, rho*u, E of p->nx doubles each); it is advanced in
 * place by nsteps steps (nsteps <= 0: the whole run of shll_steps_for(p)) with the
 * SHLL_PREC_MIXED_F64 arithmetic of shll_step, on `stream` (a cudaStream_t, NULL = default).
 * All other memory it needs lives in one 2 MiB array inside the library, which every GPU that
 * loads the library holds until the process exits; so p->nx is limited to 65536 cells (larger
 * tubes are rejected with SHLL_ERR_ARG), p->dim must be 1 and p->precision MIXED_F64, and the
 * other parameters pass the same checks as in shll_create (SHLL_ERR_ARG otherwise).  The first
 * call on each device looks up that array's device address: make it before any stream capture.
 * The address is kept for the life of the process, so do not call this entry point again on a
 * device after cudaDeviceReset() (which unloads the library's device image).
 * Every call uses the same array and leaves its contents behind, so calls that overlap on the
 * GPU (other threads, other streams) race with each other; serialise them.  Returns after the
 * work has completed. */
int shll_tube_run_static(const shll_params* p, double* d_cons, long nsteps, void* stream);

/* The autotuner for a single mixed-precision context (see shll_batch_autotune).  2D (contexts and
 * batches): the fold window (16, 32, 64 or 128 steps) and, for first order, the time steps per
 * step launch (1 or 2) are timed and chosen for the whole batch and, process-wide, for its size
 * class (state format, scheme, floor(log2 of the largest domain's cells)); shll_tuning /
 * shll_batch_tuning then report the steps per launch as the sweep length, that fold window and
 * 512-cell tiles. */
int shll_autotune(shll_ctx* ctx, int trial_steps);
int shll_tuning(shll_ctx* ctx, int* sweep_steps, int* fold_steps, int* chunk_cells);

/* Replay of captured launch sequences (no counterpart in the reference): a mixed-precision run (1D:
 * the sweep launches; 2D: the step and fold launches) is captured into a CUDA graph the second time
 * its step counts (and 1D buffer parities, 2D fold window) occur, and the graph is replayed by later
 * identical runs; a run that occurs once is launched directly.  Runs on the legacy default stream
 * are launched directly.  on = 0 launches every run directly (default 1; process-wide). */
void shll_set_graph_replay(int on);

/* Resident runs (no counterpart in the reference): a mixed-precision 1D run whose chunks fit on
 * the GPU at once (one block per multiprocessor: a tube of up to about 68000 cells at the default
 * sweep length) and share one scheme variant is one cooperative launch in which every chunk
 * waits, with a bounded wait, only for its two neighbours' previous sweep, and keeps its frame
 * and its cells' FP32 pairs on chip between the sweeps of a fold window.  Results are identical
 * to the one-launch-per-sweep schedule.  on = 0 selects that schedule for every run (default 1;
 * process-wide).  A wait that gives up makes the run return SHLL_ERR_TIMEOUT. */
void shll_set_resident(int on);

/* Pair flux of first-order mixed-precision 1D runs (no counterpart in the reference): where the
 * flow is supersonic, the reference scheme (base-c/base_shll.c:130-159, whose split gives the
 * u - a wave the negative numerical viscosity a(1 - M)/2 once M > 1) amplifies every per-step
 * rounding error by orders of magnitude.  So a chunk of cells whose own or neighbouring cells
 * exceeded Mach 0.6 at the end of a sweep (or, at the start of a run, held a pressure jump of more
 * than 1.5 times) evaluates its split fluxes, interface sums and increments of the next sweep in
 * double-FP32 arithmetic (pairs of FP32 numbers, about 48 significant bits) instead of FP32.
 * on = 0 keeps FP32 everywhere; on = 2 uses the pair flux in every chunk of every tube, first
 * and second order (the second-order scheme amplifies rounding everywhere, not only in supersonic
 * flow: this is the mode in which second-order runs meet FP64 results to L1 1e-6 on long tubes,
 * at about half the FP32 throughput) (default 1; process-wide). */
void shll_set_pair_flux(int on);

/* Cluster runs (no counterpart in the reference): a mixed-precision 1D run whose tubes share one
 * scheme variant and one chunk count of 2 to 16 runs as one launch in which each tube is a
 * thread-block cluster, the wait between its sweeps being the cluster's hardware barrier instead of
 * the resident run's neighbour progress counters (the data still passes through L2); the tubes need
 * not fit on the GPU at once.  Results are identical to the other schedules.  on = 1 enables it
 * (default 0, a measured alternative; process-wide). */
void shll_set_cluster_runs(int on);

/* Test hook (no counterpart in the reference): in resident runs the chunk with this index (chunks
 * are numbered along the tubes from 0) never publishes its progress, so its neighbours' bounded
 * waits run out and the run returns SHLL_ERR_TIMEOUT; -1 (the default) switches it off.
 * Process-wide. */
void shll_debug_stall_chunk(int chunk);

/* ---- the reference's own entry points on a process-wide default context ----
 * shll_ref_configure() chooses the problem (else base_shll.c's defaults, N = 256, F64). */
int shll_ref_configure(const shll_params* p);
shll_ctx* shll_ref_context(void);
void Allocate_and_Init_Memory(void);
void Compute_U_from_P(void);
void Compute_P_from_U(void);
void Compute_F_from_P(void);
void Update_U_from_F(void);
void Save_Results(void);
void Free_Memory(void);
/* DT of the default context (the reference's global float DT, base_shll.c:23) */
double shll_ref_dt(void);

#ifdef __cplusplus
}
#endif
#endif

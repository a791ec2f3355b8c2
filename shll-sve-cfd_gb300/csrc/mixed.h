// Mixed-precision engine (SHLL_PREC_MIXED_F64 / SHLL_PREC_MIXED_KAHAN): one or many independent
// tubes (1D) or domains (2D) advanced by FP32 perturbation-form split fluxes with compensated
// FP32 accumulation, folded into the stored state (FP64, or an FP32 pair) every sweep.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

#include "../../include/shll.h"

struct MixedState;

MixedState* mixed_create(const shll_params* p, double dtdx, double dtdy, double cv, cudaStream_t s, char* err,
                         size_t errlen);
MixedState* mixed_create_batch(const shll_params* items, int count, cudaStream_t s, char* err, size_t errlen);
void mixed_destroy(MixedState* m);
void mixed_set_stream(MixedState* m, cudaStream_t s);
// loads primitive planes (double) of item 0 (single-context use)
int mixed_load(MixedState* m, const double* prim, char* err, size_t errlen);
// loads every item of a batch from its own initial-condition descriptor
int mixed_load_all(MixedState* m, char* err, size_t errlen);
// item `item`'s state from host primitive planes (nv pointers: rho, u, [v,] T; pinned host memory
// is copied at full link speed), converted to conserved variables on the device; SHLL_ERR_ARG,
// with the state unchanged, if a cell's density or temperature is not positive
int mixed_set_item_primitives(MixedState* m, int item, const double* const* planes, char* err, size_t errlen);
// every item at once: `prim` holds, item after item, each item's planes rho, u, [v,] T (one copy
// each way, one conversion kernel per item, one synchronisation)
int mixed_set_all_primitives(MixedState* m, const double* prim, char* err, size_t errlen);
int mixed_get_all_primitives(MixedState* m, double* prim, char* err, size_t errlen);

// where one item's stored state lies (the 1D and 2D engines share the device conversions)
struct MixedPlanes {
    void* hi;        // FP64 planes, or the FP32 value planes of a pair state
    float* lo;       // FP32 compensation planes (pair state) or null
    long base;       // first cell of the item in every plane
    long plane;      // cells per plane
    long n;          // cells of the item
    int nv;          // conserved components: 3 (1D) or 4 (2D)
    bool kahan;
    double CV;       // R / (gamma - 1)
};
int mixed2d_planes(MixedState* m, int item, MixedPlanes* out);   // mixed2d.cu
const shll_params* mixed_items(MixedState* m, int* count);
// advances every item by nsteps (capped at each item's own remaining steps when nsteps < 0:
// "run to the end")
int mixed_step(MixedState* m, long nsteps, char* err, size_t errlen);
int mixed_get_primitives(MixedState* m, double* rho, double* u, double* v, double* T, char* err, size_t errlen);
int mixed_get_conserved(MixedState* m, double* planes, char* err, size_t errlen);
int mixed_totals(MixedState* m, double* out, char* err, size_t errlen);
int mixed_item_primitives(MixedState* m, int item, double* rho, double* u, double* v, double* T, char* err,
                          size_t errlen);
int mixed_item_totals(MixedState* m, int item, double* out, char* err, size_t errlen);
int mixed_item_conserved(MixedState* m, int item, double* planes, char* err, size_t errlen);
long mixed_cell_updates(const MixedState* m);
int mixed_checkpoint(MixedState* m, bool restore, char* err, size_t errlen);
int mixed_flags(MixedState* m);
int mixed_autotune(MixedState* m, int trial_steps, char* err, size_t errlen);
int mixed_tuning(MixedState* m, int item, int* sweep_steps, int* fold_steps, int* chunk_cells);
int mixed_item_flags(MixedState* m, int item);

// FP64 plane sums (reduce.cu)
cudaError_t device_plane_sums(const void* planes, int real_bits, int nv, long n, double* out, cudaStream_t s);
cudaError_t device_pair_sums(const float* hi, const float* lo, int nv, long n, double* out, cudaStream_t s);

// initial conditions (capi.cu)
void shll_ic_fill(const shll_params* p, int real_bits, double* prim);

// Plain FP64 batches (plain_batch.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

#include "../../include/shll.h"

struct PlainBatch;
PlainBatch* plain_batch_create(const shll_params* p, int count, cudaStream_t s, char* err, size_t len);
void plain_batch_destroy(PlainBatch* b);
void plain_batch_set_stream(PlainBatch* b, cudaStream_t s);
int plain_batch_load(PlainBatch* b, char* err, size_t len);
int plain_batch_run(PlainBatch* b, char* err, size_t len);
int plain_batch_flags(PlainBatch* b);
int plain_batch_item_flags(PlainBatch* b, int t);
long plain_batch_cell_updates(const PlainBatch* b);
int plain_batch_item_primitives(PlainBatch* b, int t, double* rho, double* u, double* v, double* T, char* err,
                                size_t len);
int plain_batch_item_totals(PlainBatch* b, int t, double* out, char* err, size_t len);

// shared helpers defined elsewhere
void shll_ic_fill(const shll_params* p, int real_bits, double* prim);
cudaError_t device_plane_sums(const void* planes, int real_bits, int nv, long n, double* out, cudaStream_t s);

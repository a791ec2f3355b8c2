// Kernels of the plain FP64 batches without fused multiply-add (this unit is compiled with
// -fmad=false): SHLL_PREC_F64_EXACT batch items are bit-identical to the FP64 reference build,
// as the single-problem exact path is (plain_exact.cu).
#define SHLL_PLAIN_NS plain_batch_exact_ns
#include "plain_batch_kernels.cuh"

cudaError_t plain_batch_exact_launch(int dim, int order, int nb, cudaStream_t s, const void* items, const void* blks,
                                     double* U0, double* U1, long plane, int step, int* flags) {
    using namespace plain_batch_exact_ns;
    return batch_launch(dim, order, nb, s, static_cast<const PItem*>(items), static_cast<const PBlk*>(blks), U0, U1,
                        plane, step, flags);
}

// Kernels of the plain FP64 batches, compiled once per arithmetic: plain_batch.cu (fused
// multiply-add allowed, SHLL_PREC_F64) and plain_batch_exact.cu (-fmad=false, SHLL_PREC_F64_EXACT:
// bit-identical to the FP64 reference build).  The including unit defines SHLL_PLAIN_NS.
#pragma once
#include "shll_plain.cuh"

namespace SHLL_PLAIN_NS {
struct PItem {
    long base;        // cell offset in the planes
    int nx, ny;       // ny = 1 in 1D
    int order, steps, par;
    Gas<double> g;
};

struct PBlk { int item, a, b; };  // 1D: first cell a; 2D: tile origin (a, b) = (i0, j0)

// (flag points at the item's own flag word; the kernel ORs SHLL_FLAG_NONPOSITIVE into it)
template <int ORDER>
__global__ void __launch_bounds__(T1) k_batch1(const PItem* __restrict__ items, const PBlk* __restrict__ blks,
                                               double* U0, double* U1, long plane, int step, int* flags) {
    const PBlk bk = blks[blockIdx.x];
    const PItem it = items[bk.item];
    if (step >= it.steps) return;
    const int inb = (it.par + step) & 1;
    const double* Uin = (inb ? U1 : U0) + it.base;
    double* Uout = (inb ? U0 : U1) + it.base;
    step1_block<double, ORDER>(Uin, Uout, it.nx, plane, it.g, flags + bk.item, bk.a);
}

template <int ORDER>
__global__ void __launch_bounds__(TI * TJ) k_batch2(const PItem* __restrict__ items, const PBlk* __restrict__ blks,
                                                    double* U0, double* U1, long plane, int step, int* flags) {
    const PBlk bk = blks[blockIdx.x];
    const PItem it = items[bk.item];
    if (step >= it.steps) return;
    const int inb = (it.par + step) & 1;
    const double* Uin = (inb ? U1 : U0) + it.base;
    double* Uout = (inb ? U0 : U1) + it.base;
    step2_tile<double, ORDER>(Uin, Uout, it.nx, it.ny, plane, it.g, flags + bk.item, bk.a, bk.b);
}

// one time step of the nb active blocks of one order (dim 1: k_batch1, dim 2: k_batch2)
static cudaError_t batch_launch(int dim, int order, int nb, cudaStream_t s, const PItem* items, const PBlk* blks,
                                double* U0, double* U1, long plane, int step, int* flags) {
    if (dim == 1) {
        if (order == 1) k_batch1<1><<<nb, T1, 0, s>>>(items, blks, U0, U1, plane, step, flags);
        else k_batch1<2><<<nb, T1, 0, s>>>(items, blks, U0, U1, plane, step, flags);
    } else {
        static unsigned long long attr_set = 0;  // devices on which the shared-memory size is allowed
        int dev = 0;
        cudaGetDevice(&dev);
        if (dev < 64 && !(attr_set & (1ull << dev))) {
            cudaFuncSetAttribute(k_batch2<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2<double, 1>());
            cudaFuncSetAttribute(k_batch2<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2<double, 2>());
            attr_set |= 1ull << dev;
        }
        dim3 blk(TJ, TI);
        if (order == 1) k_batch2<1><<<nb, blk, smem2<double, 1>(), s>>>(items, blks, U0, U1, plane, step, flags);
        else k_batch2<2><<<nb, blk, smem2<double, 2>(), s>>>(items, blks, U0, U1, plane, step, flags);
    }
    return cudaGetLastError();
}

}  // namespace SHLL_PLAIN_NS

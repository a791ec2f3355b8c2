// FP64 conservation sums: sum over cells of each conserved plane (mass, momentum, energy).
// Warp-shuffle + shared-memory block reduction into per-block partials, summed on the host
// in a fixed order, so the result is reproducible run to run.
#include <cuda_runtime.h>

#include <vector>

#include "mixed.h"
#include "shll_internal.h"

namespace {
constexpr int RB = 256;     // threads per block
constexpr int RGRID = 304;  // 2 blocks per SM on 152 SMs

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// value of element i of plane k; for LO != nullptr the value is hi + lo (a compensated pair)
template <typename T>
__global__ void __launch_bounds__(RB) k_plane_sums(const T* __restrict__ hi, const T* __restrict__ lo, int nv, long n,
                                                  double* __restrict__ partial) {
    __shared__ double red[RB / 32];
    for (int k = 0; k < nv; k++) {
        double s = 0.0;
        for (long i = (long)blockIdx.x * RB + threadIdx.x; i < n; i += (long)gridDim.x * RB) {
            s += (double)hi[k * n + i];
            if (lo) s += (double)lo[k * n + i];
        }
        s = warp_sum(s);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x < 32) {
            double v = threadIdx.x < RB / 32 ? red[threadIdx.x] : 0.0;
            v = warp_sum(v);
            if (threadIdx.x == 0) partial[k * gridDim.x + blockIdx.x] = v;
        }
        __syncthreads();
    }
}
}  // namespace

template <typename T>
static cudaError_t sums_t(const T* hi, const T* lo, int nv, long n, double* out, cudaStream_t s) {
    double* d = nullptr;
    cudaError_t e = cudaMallocAsync(&d, sizeof(double) * nv * RGRID, s);
    if (e != cudaSuccess) return e;
    shll_count_launches(1);
    k_plane_sums<T><<<RGRID, RB, 0, s>>>(hi, lo, nv, n, d);
    std::vector<double> h((size_t)nv * RGRID);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), d, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return e;
    for (int k = 0; k < nv; k++) {
        double t = 0.0;
        for (int b = 0; b < RGRID; b++) t += h[(size_t)k * RGRID + b];
        out[k] = t;
    }
    return cudaSuccess;
}

cudaError_t device_plane_sums(const void* planes, int real_bits, int nv, long n, double* out, cudaStream_t s) {
    if (real_bits == 32) return sums_t<float>(static_cast<const float*>(planes), nullptr, nv, n, out, s);
    return sums_t<double>(static_cast<const double*>(planes), nullptr, nv, n, out, s);
}

cudaError_t device_pair_sums(const float* hi, const float* lo, int nv, long n, double* out, cudaStream_t s) {
    return sums_t<float>(hi, lo, nv, n, out, s);
}

// Plain SHLL kernels: the reference's arithmetic, one fused launch per time step.
//
// Included by plain_fast.cu (compiled with fused multiply-add allowed: SHLL_PREC_F64) and by
// plain_exact.cu (compiled with -fmad=false: SHLL_PREC_F64_EXACT and SHLL_PREC_F32_EXACT,
// bit-identical to the reference's gcc builds).  SHLL_PLAIN_NS names the namespace.
//
// Each expression follows the reference's evaluation order and promotions:
//   Compute_P_from_U   base-c/base_shll.c:161-177, base-c/base_shll_2d.c:302-319
//   Compute_F_from_P   base-c/base_shll.c:130-159, base-c/base_shll_2d.c:239-300
//   Update_U_from_F    base-c/base_shll.c:87-128 (reflective walls), base-c/base_shll_2d.c:139-237,
//                      base-c/2nd_order_base_shll.c:203-459 (minmod slopes, outflow walls)
// D(x) widens an operand that the reference promotes to double (a double literal or sqrt()
// touches it); with REAL = double it is a no-op.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>

#include "shll_internal.h"

namespace SHLL_PLAIN_NS {

#define D(x) ((double)(x))

template <typename REAL>
struct Gas {
    REAL R, GAMMA, CV, DT_ON_DX, DT_ON_DY, alpha;
    int limiter;
};

template <typename REAL>
__host__ Gas<REAL> make_gas(const PlainArgs& a) {
    Gas<REAL> g;
    g.R = (REAL)a.R; g.GAMMA = (REAL)a.GAMMA; g.CV = (REAL)a.CV;
    g.DT_ON_DX = (REAL)a.DT_ON_DX; g.DT_ON_DY = (REAL)a.DT_ON_DY;
    g.alpha = (REAL)a.mc_alpha; g.limiter = a.limiter;
    return g;
}

// sqrt of a REAL argument as the reference evaluates it: sqrt(double) rounded to REAL.  For
// float this equals the correctly rounded sqrtf (53 >= 2*24+2, so the double rounding is exact).
__device__ __forceinline__ float sqrt_ref(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_ref(double x) { return sqrt(x); }

// ---------------- 1D ----------------
// P from U (base_shll.c:171-176); returns p1 (velocity), p2 (temperature), a (sound speed)
template <typename REAL>
__device__ __forceinline__ void prim1(const Gas<REAL>& g, REAL u0, REAL u1, REAL u2, REAL& p1, REAL& p2, REAL& a) {
    p1 = u1 / u0;
    p2 = (REAL)((D(u2 / u0) - 0.5 * D(p1) * D(p1)) / D(g.CV));
    a = sqrt_ref(g.GAMMA * g.R * p2);
}

// split fluxes (base_shll.c:134-158) from P (p0 = u0) and U
template <typename REAL>
__device__ __forceinline__ void flux1(const Gas<REAL>& g, REAL u0, REAL u1, REAL u2, REAL p1, REAL p2, REAL a,
                                      REAL fp[3], REAL fm[3]) {
    REAL M = p1 / a;
    REAL Z1 = (REAL)(0.5 * (D(M) + 1.0));
    REAL Z2 = (REAL)(0.5 * D(a) * (1.0 - D(M * M)));
    REAL Z3 = (REAL)(0.5 * (D(M) - 1.0));
    REAL P = u0 * g.R * p2;
    REAL f0 = u1, f1 = u1 * p1 + P, f2 = p1 * (u2 + P);
    fp[0] = f0 * Z1 + u0 * Z2; fp[1] = f1 * Z1 + u1 * Z2; fp[2] = f2 * Z1 + u2 * Z2;
    fm[0] = -f0 * Z3 - u0 * Z2; fm[1] = -f1 * Z3 - u1 * Z2; fm[2] = -f2 * Z3 - u2 * Z2;
}

// minmod (2nd_order_base_shll.c:191-201)
template <typename REAL>
__device__ __forceinline__ REAL minmod(REAL l, REAL r) {
    if (l * r < 0.0) return (REAL)0.0;
    return (fabs(D(l)) < fabs(D(r))) ? l : r;
}
// slope of a split flux at an interior cell: minmod, or the MC limiter of
// base-omp/2nd_order_base_shll.c:316-325
template <typename REAL>
__device__ __forceinline__ REAL slope(const Gas<REAL>& g, REAL fl, REAL fc, REAL fr) {
    if (g.limiter == 1)
        return minmod<REAL>((REAL)(0.5 * D(fr - fl)), g.alpha * minmod<REAL>(fc - fl, fr - fc));
    return minmod<REAL>(fc - fl, fr - fc);
}

constexpr int T1 = 256;  // cells per block (1D)

// One fused time step in 1D: P and split fluxes for the block's cells plus halo (in shared
// memory), slopes (order 2), then the reference's per-cell update.  Uin/Uout: 3 planes of n.
// Body of one 1D block: cells [b0, b0+T1) of a tube of n cells whose component k lives at
// U[k*stride + c].
template <typename REAL, int ORDER>
__device__ __forceinline__ void step1_block(const REAL* __restrict__ Uin, REAL* __restrict__ Uout, int n, long stride,
                                            const Gas<REAL>& g, int* __restrict__ flag, int b0) {
    constexpr int H = ORDER;
    constexpr int W = T1 + 2 * H;
    __shared__ REAL sfp[3][W], sfm[3][W];
    __shared__ REAL sdp[3][ORDER == 2 ? T1 + 2 : 1], sdm[3][ORDER == 2 ? T1 + 2 : 1];
    int bad = 0;
    for (int t = threadIdx.x; t < W; t += T1) {
        int c = b0 - H + t;
        REAL fp[3] = {0, 0, 0}, fm[3] = {0, 0, 0};
        if (c >= 0 && c < n) {
            REAL u0 = Uin[c], u1 = Uin[stride + c], u2 = Uin[2 * stride + c], p1, p2, a;
            prim1(g, u0, u1, u2, p1, p2, a);
            flux1(g, u0, u1, u2, p1, p2, a, fp, fm);
            bad |= !(u0 > (REAL)0) || !(p2 > (REAL)0);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) { sfp[k][t] = fp[k]; sfm[k][t] = fm[k]; }
    }
    __syncthreads();
    if (ORDER == 2) {
        for (int t = threadIdx.x; t < T1 + 2; t += T1) {
            int c = b0 - 1 + t, s = t + 1;  // shared index of cell c
#pragma unroll
            for (int k = 0; k < 3; k++) {
                REAL dp = 0, dm = 0;
                if (c > 0 && c < n - 1) {
                    dp = slope(g, sfp[k][s - 1], sfp[k][s], sfp[k][s + 1]);
                    dm = slope(g, sfm[k][s - 1], sfm[k][s], sfm[k][s + 1]);
                }
                sdp[k][t] = dp; sdm[k][t] = dm;
            }
        }
        __syncthreads();
    }
    const int i = b0 + threadIdx.x;
    if (bad) atomicOr(flag, SHLL_FLAG_NONPOSITIVE);
    if (i >= n) return;
    const int s = threadIdx.x + H;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        REAL fp = sfp[k][s], fm = sfm[k][s], L, Rr, u = Uin[k * stride + i];
        if (ORDER == 1) {
            const REAL sg = (k == 1) ? (REAL)1 : (REAL)-1;  // reflective wall (base_shll.c:93-110)
            if (i == 0) { L = sg * fm; Rr = sfm[k][s + 1]; }
            else if (i == n - 1) { L = sfp[k][s - 1]; Rr = sg * fp; }
            else { L = sfp[k][s - 1]; Rr = sfm[k][s + 1]; }
            u = u - g.DT_ON_DX * (fp - fm + Rr - L);
        } else {
            const int d = threadIdx.x + 1;  // slope index of cell i
            REAL Ldf, Rdf;
            if (i == 0) { L = fp; Rr = sfm[k][s + 1]; Ldf = 0; Rdf = sdm[k][d + 1]; }
            else if (i == n - 1) { L = sfp[k][s - 1]; Rr = fm; Ldf = sdp[k][d - 1]; Rdf = 0; }
            else { L = sfp[k][s - 1]; Rr = sfm[k][s + 1]; Ldf = sdp[k][d - 1]; Rdf = sdm[k][d + 1]; }
            u = u - g.DT_ON_DX * (fp - fm + Rr - L);
            u = (REAL)(D(u) - 0.5 * D(g.DT_ON_DX) * D(sdp[k][d] + sdm[k][d] - Rdf - Ldf));
        }
        Uout[k * stride + i] = u;
    }
}

template <typename REAL, int ORDER>
__global__ void __launch_bounds__(T1) k_step1(const REAL* __restrict__ Uin, REAL* __restrict__ Uout, int n,
                                              Gas<REAL> g, int* __restrict__ flag) {
    step1_block<REAL, ORDER>(Uin, Uout, n, n, g, flag, blockIdx.x * T1);
}

// ---------------- 2D ----------------
template <typename REAL>
__device__ __forceinline__ void prim2(const Gas<REAL>& g, REAL u0, REAL u1, REAL u2, REAL u3, REAL& p1, REAL& p2,
                                      REAL& p3, REAL& a) {
    p1 = u1 / u0;
    p2 = u2 / u0;
    p3 = (REAL)((D(u3 / u0) - 0.5 * D(p1 * p1 + p2 * p2)) / D(g.CV));
    a = sqrt_ref(g.GAMMA * g.R * p3);
}

// x and y split fluxes (base_shll_2d.c:243-299)
template <typename REAL>
__device__ __forceinline__ void flux2(const Gas<REAL>& g, const REAL u[4], REAL p1, REAL p2, REAL p3, REAL a,
                                      REAL fp[4], REAL fm[4], REAL hp[4], REAL hm[4]) {
    REAL P = u[0] * g.R * p3;
    REAL M = p1 / a;
    REAL Z1 = (REAL)(0.5 * (D(M) + 1.0));
    REAL Z2 = (REAL)(0.5 * D(a) * (1.0 - D(M * M)));
    REAL Z3 = (REAL)(0.5 * (D(M) - 1.0));
    REAL f[4] = {u[1], u[1] * p1 + P, u[1] * p2, p1 * (u[3] + P)};
#pragma unroll
    for (int k = 0; k < 4; k++) { fp[k] = f[k] * Z1 + u[k] * Z2; fm[k] = -f[k] * Z3 - u[k] * Z2; }
    M = p2 / a;
    Z1 = (REAL)(0.5 * (D(M) + 1.0));
    Z2 = (REAL)(0.5 * D(a) * (1.0 - D(M * M)));
    Z3 = (REAL)(0.5 * (D(M) - 1.0));
    REAL h[4] = {u[2], u[2] * p1, u[2] * p2 + P, p2 * (u[3] + P)};
#pragma unroll
    for (int k = 0; k < 4; k++) { hp[k] = h[k] * Z1 + u[k] * Z2; hm[k] = -h[k] * Z3 - u[k] * Z2; }
}

constexpr int TJ = 32;  // tile extent along j (contiguous, threadIdx.x)
constexpr int TI = 8;   // tile extent along i (threadIdx.y)

template <int ORDER>
struct Tile2 {
    static constexpr int H = ORDER;
    static constexpr int WI = TI + 2 * H, WJ = TJ + 2 * H, CELLS = WI * WJ;
};

template <typename REAL, int ORDER>
constexpr size_t smem2() {
    using TL = Tile2<ORDER>;
    size_t flux = (size_t)16 * TL::CELLS * sizeof(REAL);
    size_t slopes = ORDER == 2 ? (size_t)8 * ((TI + 2) * TJ + TI * (TJ + 2)) * sizeof(REAL) : 0;
    return flux + slopes;
}

// One fused 2D time step on a TI x TJ tile.  Shared memory holds fp, fm, hp, hm (4 components
// each) for the tile plus an ORDER-wide halo, then (order 2) the x and y slopes.
// Body of one 2D tile with origin (i0, j0) of an nx x ny domain whose component k lives at
// U[k*stride + i*ny + j].
template <typename REAL, int ORDER>
__device__ __forceinline__ void step2_tile(const REAL* __restrict__ Uin, REAL* __restrict__ Uout, int nx, int ny,
                                           long stride, const Gas<REAL>& g, int* __restrict__ flag, int i0, int j0) {
    using TL = Tile2<ORDER>;
    constexpr int H = TL::H, WJ = TL::WJ, CELLS = TL::CELLS;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    REAL* sf = reinterpret_cast<REAL*>(smem_raw);      // [16][CELLS]: fp0..3 fm0..3 hp0..3 hm0..3
    REAL* sd = sf + 16 * CELLS;                          // order 2 slopes
    constexpr int NXS = (TI + 2) * TJ, NYS = TI * (TJ + 2);
    const long n = stride;
    const int tid = threadIdx.y * TJ + threadIdx.x;
    int bad = 0;
    for (int t = tid; t < CELLS; t += TI * TJ) {
        int li = t / WJ, lj = t % WJ;
        int i = i0 - H + li, j = j0 - H + lj;
        REAL fp[4] = {0, 0, 0, 0}, fm[4] = {0, 0, 0, 0}, hp[4] = {0, 0, 0, 0}, hm[4] = {0, 0, 0, 0};
        if (i >= 0 && i < nx && j >= 0 && j < ny) {
            int c = i * ny + j;
            REAL u[4] = {Uin[c], Uin[n + c], Uin[2 * n + c], Uin[3 * n + c]}, p1, p2, p3, a;
            prim2(g, u[0], u[1], u[2], u[3], p1, p2, p3, a);
            flux2(g, u, p1, p2, p3, a, fp, fm, hp, hm);
            bad |= !(u[0] > (REAL)0) || !(p3 > (REAL)0);
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            sf[k * CELLS + t] = fp[k]; sf[(4 + k) * CELLS + t] = fm[k];
            sf[(8 + k) * CELLS + t] = hp[k]; sf[(12 + k) * CELLS + t] = hm[k];
        }
    }
    __syncthreads();
    auto F = [&](int q, int k, int li, int lj) -> REAL { return sf[(q * 4 + k) * CELLS + li * WJ + lj]; };
    if (ORDER == 2) {
        // x slopes for local rows -1..TI (cells i0-1..i0+TI), cols 0..TJ-1
        for (int t = tid; t < NXS; t += TI * TJ) {
            int r = t / TJ, lj = t % TJ;
            int i = i0 - 1 + r, j = j0 + lj, li = r - 1 + H, ljj = lj + H;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                REAL dp = 0, dm = 0;
                if (i > 0 && i < nx - 1 && j < ny) {
                    dp = slope(g, F(0, k, li - 1, ljj), F(0, k, li, ljj), F(0, k, li + 1, ljj));
                    dm = slope(g, F(1, k, li - 1, ljj), F(1, k, li, ljj), F(1, k, li + 1, ljj));
                }
                sd[k * NXS + t] = dp; sd[(4 + k) * NXS + t] = dm;
            }
        }
        // y slopes for rows 0..TI-1, cols -1..TJ
        for (int t = tid; t < NYS; t += TI * TJ) {
            int r = t / (TJ + 2), c2 = t % (TJ + 2);
            int i = i0 + r, j = j0 - 1 + c2, li = r + H, lj = c2 - 1 + H;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                REAL dp = 0, dm = 0;
                if (j > 0 && j < ny - 1 && i < nx) {
                    dp = slope(g, F(2, k, li, lj - 1), F(2, k, li, lj), F(2, k, li, lj + 1));
                    dm = slope(g, F(3, k, li, lj - 1), F(3, k, li, lj), F(3, k, li, lj + 1));
                }
                sd[8 * NXS + k * NYS + t] = dp; sd[8 * NXS + (4 + k) * NYS + t] = dm;
            }
        }
        __syncthreads();
    }
    if (bad) atomicOr(flag, SHLL_FLAG_NONPOSITIVE);
    const int i = i0 + threadIdx.y, j = j0 + threadIdx.x;
    if (i >= nx || j >= ny) return;
    const int c = i * ny + j, li = threadIdx.y + H, lj = threadIdx.x + H;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        REAL u = Uin[k * n + c];
        REAL fp = F(0, k, li, lj), fm = F(1, k, li, lj), hp = F(2, k, li, lj), hm = F(3, k, li, lj);
        if (ORDER == 1) {
            // reflective walls: x flips components 0,2,3; y flips 0,1,3 (base_shll_2d.c:150-216)
            const REAL sx = (k == 1) ? (REAL)1 : (REAL)-1, sy = (k == 2) ? (REAL)1 : (REAL)-1;
            REAL L, Rr, B, Tt;
            if (i == 0) { L = sx * fm; Rr = F(1, k, li + 1, lj); }
            else if (i == nx - 1) { L = F(0, k, li - 1, lj); Rr = sx * fp; }
            else { L = F(0, k, li - 1, lj); Rr = F(1, k, li + 1, lj); }
            if (j == 0) { B = sy * hm; Tt = F(3, k, li, lj + 1); }
            else if (j == ny - 1) { B = F(2, k, li, lj - 1); Tt = sy * hp; }
            else { B = F(2, k, li, lj - 1); Tt = F(3, k, li, lj + 1); }
            u = u - g.DT_ON_DX * (fp - fm + Rr - L);
            u = u - g.DT_ON_DY * (hp - hm + Tt - B);
        } else {
            // outflow walls, slopes zero on edge cells (2nd_order_base_shll.c:210-458)
            auto DX_ = [&](int q, int r) -> REAL { return sd[(q * 4 + k) * NXS + r * TJ + threadIdx.x]; };
            auto DY_ = [&](int q, int cc) -> REAL {
                return sd[8 * NXS + (q * 4 + k) * NYS + threadIdx.y * (TJ + 2) + cc];
            };
            const int r = threadIdx.y + 1, cc = threadIdx.x + 1;
            REAL L, Rr, Ldf, Rdf, B, Tt, Bdf, Tdf;
            if (i == 0) { L = fp; Rr = F(1, k, li + 1, lj); Ldf = 0; Rdf = DX_(1, r + 1); }
            else if (i == nx - 1) { L = F(0, k, li - 1, lj); Rr = fm; Ldf = DX_(0, r - 1); Rdf = 0; }
            else { L = F(0, k, li - 1, lj); Rr = F(1, k, li + 1, lj); Ldf = DX_(0, r - 1); Rdf = DX_(1, r + 1); }
            if (j == 0) { B = hp; Tt = F(3, k, li, lj + 1); Bdf = 0; Tdf = DY_(1, cc + 1); }
            else if (j == ny - 1) { B = F(2, k, li, lj - 1); Tt = hm; Bdf = DY_(0, cc - 1); Tdf = 0; }
            else { B = F(2, k, li, lj - 1); Tt = F(3, k, li, lj + 1); Bdf = DY_(0, cc - 1); Tdf = DY_(1, cc + 1); }
            u = u - g.DT_ON_DX * (fp - fm + Rr - L);
            u = (REAL)(D(u) - 0.5 * D(g.DT_ON_DX) * D(DX_(0, r) + DX_(1, r) - Rdf - Ldf));
            u = u - g.DT_ON_DY * (hp - hm + Tt - B);
            u = (REAL)(D(u) - 0.5 * D(g.DT_ON_DY) * D(DY_(0, cc) + DY_(1, cc) - Tdf - Bdf));
        }
        Uout[k * n + c] = u;
    }
}

template <typename REAL, int ORDER>
__global__ void __launch_bounds__(TI * TJ) k_step2(const REAL* __restrict__ Uin, REAL* __restrict__ Uout, int nx,
                                                   int ny, Gas<REAL> g, int* __restrict__ flag) {
    step2_tile<REAL, ORDER>(Uin, Uout, nx, ny, (long)nx * ny, g, flag, blockIdx.y * TI, blockIdx.x * TJ);
}

// ---------------- staged kernels (the reference's separate stages) ----------------
// Compute_U_from_P: base_shll.c:76-80 / base_shll_2d.c:126-131.  P: nv planes (+ a plane).
template <typename REAL>
__global__ void k_u_from_p(const REAL* __restrict__ P, REAL* __restrict__ U, long n, int dim, Gas<REAL> g) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        if (dim == 1) {
            REAL p0 = P[c], p1 = P[n + c], p2 = P[2 * n + c];
            U[c] = p0; U[n + c] = p0 * p1;
            U[2 * n + c] = (REAL)(D(p0) * (D(p2 * g.CV) + 0.5 * D(p1) * D(p1)));
        } else {
            REAL p0 = P[c], p1 = P[n + c], p2 = P[2 * n + c], p3 = P[3 * n + c];
            U[c] = p0; U[n + c] = p0 * p1; U[2 * n + c] = p0 * p2;
            U[3 * n + c] = (REAL)(D(p0) * (D(p3 * g.CV) + 0.5 * D(p1 * p1 + p2 * p2)));
        }
    }
}

// Compute_P_from_U: P planes rho, u, [v,] T and the sound-speed plane a after them.
template <typename REAL>
__global__ void k_p_from_u(const REAL* __restrict__ U, REAL* __restrict__ P, long n, int dim, Gas<REAL> g,
                           int* __restrict__ flag) {
    int bad = 0;
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        if (dim == 1) {
            REAL u0 = U[c], p1, p2, a;
            prim1(g, u0, U[n + c], U[2 * n + c], p1, p2, a);
            P[c] = u0; P[n + c] = p1; P[2 * n + c] = p2; P[3 * n + c] = a;
            bad |= !(u0 > (REAL)0) || !(p2 > (REAL)0);
        } else {
            REAL u0 = U[c], p1, p2, p3, a;
            prim2(g, u0, U[n + c], U[2 * n + c], U[3 * n + c], p1, p2, p3, a);
            P[c] = u0; P[n + c] = p1; P[2 * n + c] = p2; P[3 * n + c] = p3; P[4 * n + c] = a;
            bad |= !(u0 > (REAL)0) || !(p3 > (REAL)0);
        }
    }
    if (bad) atomicOr(flag, SHLL_FLAG_NONPOSITIVE);
}

// Compute_F_from_P from the stored P (and its a plane) and U, as the reference reads both.
template <typename REAL>
__global__ void k_f_from_p(const REAL* __restrict__ U, const REAL* __restrict__ P, REAL* __restrict__ fp,
                           REAL* __restrict__ fm, REAL* __restrict__ hp, REAL* __restrict__ hm, long n, int dim,
                           Gas<REAL> g) {
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        if (dim == 1) {
            REAL a[3], b[3];
            flux1(g, U[c], U[n + c], U[2 * n + c], P[n + c], P[2 * n + c], P[3 * n + c], a, b);
            for (int k = 0; k < 3; k++) { fp[k * n + c] = a[k]; fm[k * n + c] = b[k]; }
        } else {
            REAL u[4] = {U[c], U[n + c], U[2 * n + c], U[3 * n + c]}, a[4], b[4], e[4], f[4];
            // the reference evaluates P = p0*R*p3 with p0 from the P array (equal to u0)
            flux2(g, u, P[n + c], P[2 * n + c], P[3 * n + c], P[4 * n + c], a, b, e, f);
            for (int k = 0; k < 4; k++) {
                fp[k * n + c] = a[k]; fm[k * n + c] = b[k]; hp[k * n + c] = e[k]; hm[k * n + c] = f[k];
            }
        }
    }
}

// Update_U_from_F from stored split-flux planes (in place: each cell reads only its own U).
template <typename REAL>
__global__ void k_update_staged(REAL* __restrict__ U, const REAL* __restrict__ fp, const REAL* __restrict__ fm,
                                const REAL* __restrict__ hp, const REAL* __restrict__ hm, int nx, int ny, int dim,
                                int order, Gas<REAL> g) {
    const long n = (long)nx * ny;
    const int nv = dim == 2 ? 4 : 3, sx_ = ny;  // x stride (1D: ny = 1)
    for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        const int i = (int)(c / ny), j = (int)(c % ny);
        for (int k = 0; k < nv; k++) {
            const REAL* Fp = fp + k * n; const REAL* Fm = fm + k * n;
            REAL u = U[k * n + c];
            if (order == 1) {
                const REAL sx = (k == 1) ? (REAL)1 : (REAL)-1;
                REAL L, Rr;
                if (i == 0) { L = sx * Fm[c]; Rr = Fm[c + sx_]; }
                else if (i == nx - 1) { L = Fp[c - sx_]; Rr = sx * Fp[c]; }
                else { L = Fp[c - sx_]; Rr = Fm[c + sx_]; }
                u = u - g.DT_ON_DX * (Fp[c] - Fm[c] + Rr - L);
                if (dim == 2) {
                    const REAL* Hp = hp + k * n; const REAL* Hm = hm + k * n;
                    const REAL sy = (k == 2) ? (REAL)1 : (REAL)-1;
                    REAL B, Tt;
                    if (j == 0) { B = sy * Hm[c]; Tt = Hm[c + 1]; }
                    else if (j == ny - 1) { B = Hp[c - 1]; Tt = sy * Hp[c]; }
                    else { B = Hp[c - 1]; Tt = Hm[c + 1]; }
                    u = u - g.DT_ON_DY * (Hp[c] - Hm[c] + Tt - B);
                }
            } else {
                auto sl = [&](const REAL* f, long cc, int ii, int st, int nn) -> REAL {
                    if (ii <= 0 || ii >= nn - 1) return (REAL)0;
                    return slope(g, f[cc - st], f[cc], f[cc + st]);
                };
                REAL L, Rr, Ldf, Rdf;
                if (i == 0) { L = Fp[c]; Rr = Fm[c + sx_]; Ldf = 0; Rdf = sl(Fm, c + sx_, i + 1, sx_, nx); }
                else if (i == nx - 1) { L = Fp[c - sx_]; Rr = Fm[c]; Ldf = sl(Fp, c - sx_, i - 1, sx_, nx); Rdf = 0; }
                else {
                    L = Fp[c - sx_]; Rr = Fm[c + sx_];
                    Ldf = sl(Fp, c - sx_, i - 1, sx_, nx); Rdf = sl(Fm, c + sx_, i + 1, sx_, nx);
                }
                u = u - g.DT_ON_DX * (Fp[c] - Fm[c] + Rr - L);
                u = (REAL)(D(u) - 0.5 * D(g.DT_ON_DX) * D(sl(Fp, c, i, sx_, nx) + sl(Fm, c, i, sx_, nx) - Rdf - Ldf));
                if (dim == 2) {
                    const REAL* Hp = hp + k * n; const REAL* Hm = hm + k * n;
                    REAL B, Tt, Bdf, Tdf;
                    if (j == 0) { B = Hp[c]; Tt = Hm[c + 1]; Bdf = 0; Tdf = sl(Hm, c + 1, j + 1, 1, ny); }
                    else if (j == ny - 1) { B = Hp[c - 1]; Tt = Hm[c]; Bdf = sl(Hp, c - 1, j - 1, 1, ny); Tdf = 0; }
                    else {
                        B = Hp[c - 1]; Tt = Hm[c + 1];
                        Bdf = sl(Hp, c - 1, j - 1, 1, ny); Tdf = sl(Hm, c + 1, j + 1, 1, ny);
                    }
                    u = u - g.DT_ON_DY * (Hp[c] - Hm[c] + Tt - B);
                    u = (REAL)(D(u) - 0.5 * D(g.DT_ON_DY) * D(sl(Hp, c, j, 1, ny) + sl(Hm, c, j, 1, ny) - Tdf - Bdf));
                }
            }
            U[k * n + c] = u;
        }
    }
}

#undef D

// ---------------- host launchers ----------------
template <typename REAL>
static cudaError_t step_t(const PlainArgs& a) {
    shll_count_launches(1);
    Gas<REAL> g = make_gas<REAL>(a);
    const REAL* Uin = static_cast<const REAL*>(a.Uin);
    REAL* Uout = static_cast<REAL*>(a.Uout);
    if (a.dim == 1) {
        dim3 grid((a.nx + T1 - 1) / T1);
        if (a.order == 1) k_step1<REAL, 1><<<grid, T1, 0, a.stream>>>(Uin, Uout, a.nx, g, a.flag);
        else k_step1<REAL, 2><<<grid, T1, 0, a.stream>>>(Uin, Uout, a.nx, g, a.flag);
    } else {
        dim3 grid((a.ny + TJ - 1) / TJ, (a.nx + TI - 1) / TI), block(TJ, TI);
        if (a.order == 1) {
            constexpr size_t sm = smem2<REAL, 1>();
            cudaFuncSetAttribute(k_step2<REAL, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            k_step2<REAL, 1><<<grid, block, sm, a.stream>>>(Uin, Uout, a.nx, a.ny, g, a.flag);
        } else {
            constexpr size_t sm = smem2<REAL, 2>();
            cudaFuncSetAttribute(k_step2<REAL, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            k_step2<REAL, 2><<<grid, block, sm, a.stream>>>(Uin, Uout, a.nx, a.ny, g, a.flag);
        }
    }
    return cudaGetLastError();
}

template <typename REAL>
static cudaError_t stage_t(const PlainArgs& a, int which) {
    shll_count_launches(1);
    Gas<REAL> g = make_gas<REAL>(a);
    const long n = (long)a.nx * (a.dim == 2 ? a.ny : 1);
    const int threads = 256;
    int blocks = (int)std::min<long>((n + threads - 1) / threads, 152L * 16);
    REAL* U = static_cast<REAL*>(a.Uout);
    REAL* P = static_cast<REAL*>(a.P);
    switch (which) {
        case STAGE_U_FROM_P: k_u_from_p<REAL><<<blocks, threads, 0, a.stream>>>(P, U, n, a.dim, g); break;
        case STAGE_P_FROM_U: k_p_from_u<REAL><<<blocks, threads, 0, a.stream>>>(U, P, n, a.dim, g, a.flag); break;
        case STAGE_F_FROM_P:
            k_f_from_p<REAL><<<blocks, threads, 0, a.stream>>>(U, P, static_cast<REAL*>(a.fp), static_cast<REAL*>(a.fm),
                                                             static_cast<REAL*>(a.hp), static_cast<REAL*>(a.hm), n,
                                                             a.dim, g);
            break;
        case STAGE_UPDATE:
            k_update_staged<REAL><<<blocks, threads, 0, a.stream>>>(
                U, static_cast<const REAL*>(a.fp), static_cast<const REAL*>(a.fm), static_cast<const REAL*>(a.hp),
                static_cast<const REAL*>(a.hm), a.nx, a.dim == 2 ? a.ny : 1, a.dim, a.order, g);
            break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

}  // namespace SHLL_PLAIN_NS

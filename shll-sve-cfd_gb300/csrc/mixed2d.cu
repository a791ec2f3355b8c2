// Mixed-precision 2D SHLL engine (first order, reflective walls): FP32 split fluxes in
// perturbation form, state in FP64 (SHLL_PREC_MIXED_F64) or as an FP32 value + compensation
// pair (SHLL_PREC_MIXED_KAHAN), one launch per time step over every tile of every domain.
//
// The arithmetic is that of base-c/base_shll_2d.c:139-300 re-associated as interface fluxes:
// cell (i,j) gains lam_x (F_{i-1/2} - F_{i+1/2}) + lam_y (H_{j-1/2} - H_{j+1/2}), with
// F_{i+1/2} = fp_i + fm_{i+1} and the reflective walls of base_shll_2d.c:150-216 (x walls flip
// components 0,2,3 of the split flux, y walls 0,1,3, so the wall flux is (0, 2 fm1, 0, 0) at
// i = 0, (0, 2 fp1, 0, 0) at i = nx-1, (0, 0, 2 hm2, 0) at j = 0 and (0, 0, 2 hp2, 0) at j = ny-1).
//
//   * A tile (16 x 32 cells, one CTA) has one frame: the FP64 state of its centre cell at the start
//     of the step and the split-flux coefficients derived from it.  The split fluxes of the tile's
//     cells and of its one-cell halo are evaluated in FP32 as deviations from the frame
//     (mixed_common.cuh), so rounding scales with |U - U*|.
//   * Inside a tile both cells of an interface add the same FP32 term lam*Delta with opposite
//     signs.  Neighbouring tiles evaluate their shared interfaces in different frames; each tile
//     records the full flux it applied on its edges, and at the next step the east/north tile's
//     edge cells receive lam*(F_west/south tile - F_own), so the west/south value is the one that
//     counts and mass, momentum and energy are conserved to the rounding of the state.
//   * The four interface terms of a cell are summed exactly as an FP32 pair (TwoSum) and added to
//     the state once per step (FP64 add, or FP32-pair add).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "mixed.h"
#include "mixed_common.cuh"
#include "shll_internal.h"

cudaStream_t mixed_stream(MixedState* m);
int* mixed_flag_ptr(MixedState* m);
int* mixed_item_flags_ptr(MixedState* m);
const shll_params* mixed_items(MixedState* m, int* count);
void** mixed_d2_slot(MixedState* m);
bool mixed_is_kahan(MixedState* m);
void mixed_add_updates(MixedState* m, long u);
void mixed2d_detach(MixedState* m);

namespace {

constexpr int TI = 16;           // tile rows (x, the slow index)
constexpr int TJ = 32;           // tile columns (y, contiguous)
constexpr int NT = TI * TJ;      // threads per CTA, one cell each
constexpr int WI = TI + 2, WJ = TJ + 2;

struct Dom2 {
    long base;                // cell offset of the domain in the planes
    int nx, ny, tiles_i, tiles_j;
    long ex_base, ey_base;    // first edge entry of this domain in the x / y edge buffers
    int steps, par;           // steps of the current run; buffer holding the state at its start
    double gamma, R, CV, lamx, lamy;
};

struct TileD { int dom, ti, tj; };

// one edge interface: the flux lam*F applied by the west/south tile (side 0) and by the
// east/north tile (side 1), four components each
struct Edge { double s[2][4]; };

struct Frame2 {
    double U[4], Fx[4], Fy[4];
    double fmS1, fpS1, hmS2, hpS2;   // wall split fluxes (reflective walls)
    AnchorCoef cx, cy;               // coefficients for the x and y split fluxes
    float Uh[4], Ul[4];
};

__device__ void make_frame2(Frame2& f, const double U[4], const Dom2& d) {
    const double rho = U[0], m = U[1], nn = U[2], E = U[3];
    const double u = m / rho, v = nn / rho, e = E / rho;
    const double T = (e - 0.5 * (u * u + v * v)) / d.CV;
    const double a = sqrt(d.gamma * d.R * T);
    const double P = rho * d.R * T;
    const double Fx[4] = {m, m * u + P, m * v, u * (E + P)};
    const double Fy[4] = {nn, nn * u, nn * v + P, v * (E + P)};
    const double Mx = u / a, My = v / a;
    const double Z1x = 0.5 * (Mx + 1.0), Z2x = 0.5 * a * (1.0 - Mx * Mx), Z3x = 0.5 * (Mx - 1.0);
    const double Z1y = 0.5 * (My + 1.0), Z2y = 0.5 * a * (1.0 - My * My), Z3y = 0.5 * (My - 1.0);
    for (int k = 0; k < 4; k++) {
        f.U[k] = U[k]; f.Fx[k] = Fx[k]; f.Fy[k] = Fy[k];
        f.Uh[k] = (float)U[k];
        f.Ul[k] = (float)(U[k] - (double)f.Uh[k]);
        f.cx.F[k] = (float)Fx[k]; f.cy.F[k] = (float)Fy[k];
        f.cx.Uf[k] = f.cy.Uf[k] = (float)U[k];
    }
    f.fpS1 = Fx[1] * Z1x + m * Z2x;
    f.fmS1 = -Fx[1] * Z3x - m * Z2x;
    f.hpS2 = Fy[2] * Z1y + nn * Z2y;
    f.hmS2 = -Fy[2] * Z3y - nn * Z2y;
    AnchorCoef* c[2] = {&f.cx, &f.cy};
    for (int q = 0; q < 2; q++) {
        c[q]->rho = (float)rho; c[q]->u = (float)u; c[q]->v = (float)v; c[q]->e = (float)e;
        c[q]->T = (float)T; c[q]->a = (float)a; c[q]->P = (float)P;
        c[q]->gR = (float)(d.gamma * d.R); c[q]->R = (float)d.R; c[q]->cvinv = (float)(1.0 / d.CV);
    }
    f.cx.M = (float)Mx; f.cx.Z1 = (float)Z1x; f.cx.Z2 = (float)Z2x;
    f.cy.M = (float)My; f.cy.Z1 = (float)Z1y; f.cy.Z2 = (float)Z2y;
}

// 2D split-flux deviations of a cell with conserved deviation d = (drho, dm, dn, dE):
// x fluxes (dfp, dfm) with M = u/a and y fluxes (dhp, dhm) with M = v/a (base_shll_2d.c:239-300)
__device__ __forceinline__ void dflux2(const AnchorCoef& cx, const AnchorCoef& cy, const float d[4], float dfp[4],
                                       float dfm[4], float dhp[4], float dhm[4]) {
    const float drho = d[0], dm = d[1], dn = d[2], dE = d[3];
    const float rho = __fadd_rn(cx.rho, drho);
    const float r = fast_rcp(rho);
    const float du = __fmul_rn(__fmaf_rn(-cx.u, drho, dm), r);
    const float dv = __fmul_rn(__fmaf_rn(-cx.v, drho, dn), r);
    const float u = __fadd_rn(cx.u, du), v = __fadd_rn(cx.v, dv);
    const float de = __fmul_rn(__fmaf_rn(-cx.e, drho, dE), r);
    const float ke = __fmaf_rn(__fadd_rn(u, cx.u), du, __fmul_rn(__fadd_rn(v, cx.v), dv));  // d(u^2+v^2)
    const float dT = __fmul_rn(__fmaf_rn(-0.5f, ke, de), cx.cvinv);
    const float T = __fadd_rn(cx.T, dT);
    const float gRT = __fmul_rn(cx.gR, T);
    const float ainv = rsqrtf(gRT);
    const float a = __fmul_rn(gRT, ainv);
    const float da = __fmul_rn(__fmul_rn(cx.gR, dT), fast_rcp(__fadd_rn(a, cx.a)));
    const float dP = __fmul_rn(cx.R, __fmaf_rn(drho, T, __fmul_rn(cx.rho, dT)));
    const float P = __fadd_rn(cx.P, dP);
    const float E = __fadd_rn(cx.Uf[3], dE);
    const float EP = __fadd_rn(E, P), dEP = __fadd_rn(dE, dP);
    // x direction
    {
        const float dM = __fmul_rn(__fmaf_rn(-cx.M, da, du), ainv);
        const float M = __fadd_rn(cx.M, dM);
        const float dZ1 = __fmul_rn(0.5f, dM);
        const float Z1 = __fadd_rn(cx.Z1, dZ1), Z3 = __fadd_rn(Z1, -1.0f);
        const float dZ2 = __fmul_rn(0.5f, __fmaf_rn(da, __fmaf_rn(-M, M, 1.0f), -__fmul_rn(__fmul_rn(cx.a, __fadd_rn(M, cx.M)), dM)));
        const float Z2 = __fadd_rn(cx.Z2, dZ2);
        float dF[4];
        dF[0] = dm;
        dF[1] = __fadd_rn(__fmaf_rn(dm, u, __fmul_rn(cx.Uf[1], du)), dP);
        dF[2] = __fmaf_rn(dm, v, __fmul_rn(cx.Uf[1], dv));
        dF[3] = __fmaf_rn(du, EP, __fmul_rn(cx.u, dEP));
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float a1 = __fmaf_rn(dF[k], Z1, __fmul_rn(cx.F[k], dZ1));
            const float a2 = __fmaf_rn(d[k], Z2, __fmul_rn(cx.Uf[k], dZ2));
            const float a3 = __fmaf_rn(dF[k], Z3, __fmul_rn(cx.F[k], dZ1));
            dfp[k] = __fadd_rn(a1, a2);
            dfm[k] = -__fadd_rn(a3, a2);
        }
    }
    // y direction
    {
        const float dM = __fmul_rn(__fmaf_rn(-cy.M, da, dv), ainv);
        const float M = __fadd_rn(cy.M, dM);
        const float dZ1 = __fmul_rn(0.5f, dM);
        const float Z1 = __fadd_rn(cy.Z1, dZ1), Z3 = __fadd_rn(Z1, -1.0f);
        const float dZ2 = __fmul_rn(0.5f, __fmaf_rn(da, __fmaf_rn(-M, M, 1.0f), -__fmul_rn(__fmul_rn(cy.a, __fadd_rn(M, cy.M)), dM)));
        const float Z2 = __fadd_rn(cy.Z2, dZ2);
        float dH[4];
        dH[0] = dn;
        dH[1] = __fmaf_rn(dn, u, __fmul_rn(cy.Uf[2], du));
        dH[2] = __fadd_rn(__fmaf_rn(dn, v, __fmul_rn(cy.Uf[2], dv)), dP);
        dH[3] = __fmaf_rn(dv, EP, __fmul_rn(cy.v, dEP));
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float a1 = __fmaf_rn(dH[k], Z1, __fmul_rn(cy.F[k], dZ1));
            const float a2 = __fmaf_rn(d[k], Z2, __fmul_rn(cy.Uf[k], dZ2));
            const float a3 = __fmaf_rn(dH[k], Z3, __fmul_rn(cy.F[k], dZ1));
            dhp[k] = __fadd_rn(a1, a2);
            dhm[k] = -__fadd_rn(a3, a2);
        }
    }
}

struct Args2 {
    const Dom2* doms;
    const TileD* tiles;
    void* hi[2];
    float* lo[2];
    Edge* ex[2];     // x edge buffers by step parity
    Edge* ey[2];
    long plane;
    int step;
    int* flag;
    int* item_flags;
};

template <bool KAHAN>
__device__ __forceinline__ double load2(const void* hi, const float* lo, long idx) {
    if (KAHAN) return (double)static_cast<const float*>(hi)[idx] + (double)lo[idx];
    return static_cast<const double*>(hi)[idx];
}

// boundary correction owed to cell (i, j) by the previous step (zero on the first step)
__device__ __forceinline__ void cell_correction(const Args2& A, const Dom2& D, int i, int j, double c[4]) {
    c[0] = c[1] = c[2] = c[3] = 0.0;
    if (A.step == 0) return;
    const int pp = (A.step - 1) & 1;
    if (i > 0 && i % TI == 0) {
        const Edge& e = (pp ? A.ex[1] : A.ex[0])[D.ex_base + (long)(i / TI - 1) * D.ny + j];
        for (int k = 0; k < 4; k++) c[k] += e.s[0][k] - e.s[1][k];
    }
    if (j > 0 && j % TJ == 0) {
        const Edge& e = (pp ? A.ey[1] : A.ey[0])[D.ey_base + (long)(j / TJ - 1) * D.nx + i];
        for (int k = 0; k < 4; k++) c[k] += e.s[0][k] - e.s[1][k];
    }
}

// (th, tl) = lam * x as an FP32 pair (exact when lam is an FP32 power of two)
__device__ __forceinline__ void lam_mul(float lh, float ll, float x, float& th, float& tl) {
    th = __fmul_rn(lh, x);
    tl = __fadd_rn(__fmaf_rn(lh, x, -th), __fmul_rn(ll, x));
}

struct Smem2 {
    Frame2 fr;
    float f[16][WI * WJ];   // dfp0..3, dfm0..3, dhp0..3, dhm0..3 of the window (tile + 1-cell halo)
    float wc[4][4][2];      // constant wall terms: [west, east, south, north][comp][pair]
};

template <bool KAHAN>
__global__ void __launch_bounds__(NT) k_step2d(Args2 A) {
    __shared__ Smem2 S;
    const TileD tile = A.tiles[blockIdx.x];
    const Dom2 D = A.doms[tile.dom];
    if (A.step >= D.steps) return;
    const int tid = threadIdx.x;
    const int i0 = tile.ti * TI, j0 = tile.tj * TJ;
    const int hi_i = min(TI, D.nx - i0), hi_j = min(TJ, D.ny - j0);  // tile extent
    const int inb = (D.par + A.step) & 1;
    const void* hin = inb ? A.hi[1] : A.hi[0];
    const float* lin = inb ? A.lo[1] : A.lo[0];
    void* hout = inb ? A.hi[0] : A.hi[1];
    float* lout = inb ? A.lo[0] : A.lo[1];
    const long P = A.plane;
    const long base = D.base;
    const float lxh = (float)D.lamx, lxl = (float)(D.lamx - (double)lxh);
    const float lyh = (float)D.lamy, lyl = (float)(D.lamy - (double)lyh);

    if (tid == 0) {
        const int ia = i0 + hi_i / 2, ja = j0 + hi_j / 2;
        double c[4], U[4];
        cell_correction(A, D, ia, ja, c);
        for (int k = 0; k < 4; k++) U[k] = load2<KAHAN>(hin, lin, k * P + base + (long)ia * D.ny + ja) + c[k];
        make_frame2(S.fr, U, D);
    }
    __syncthreads();
    if (tid < 16) {
        // constant wall terms: lam*(W_const - Fref) (west/south), lam*(Fref - W_const) (east/north)
        const int w = tid / 4, k = tid % 4;
        const Frame2& f = S.fr;
        double v;
        if (w == 0) v = k == 1 ? D.lamx * (2.0 * f.fmS1 - f.Fx[1]) : -D.lamx * f.Fx[k];
        else if (w == 1) v = k == 1 ? D.lamx * (f.Fx[1] - 2.0 * f.fpS1) : D.lamx * f.Fx[k];
        else if (w == 2) v = k == 2 ? D.lamy * (2.0 * f.hmS2 - f.Fy[2]) : -D.lamy * f.Fy[k];
        else v = k == 2 ? D.lamy * (f.Fy[2] - 2.0 * f.hpS2) : D.lamy * f.Fy[k];
        split2(v, S.wc[w][k][0], S.wc[w][k][1]);
    }
    // ---- split-flux deviations of the tile and its halo ----
    const int li = tid / TJ, lj = tid % TJ;          // own cell, tile coordinates
    const int i = i0 + li, j = j0 + lj;
    const bool own = li < hi_i && lj < hi_j;
    float Uh[4] = {0, 0, 0, 0}, Ul[4] = {0, 0, 0, 0};  // own state (KAHAN pair)
    double Ud[4] = {0, 0, 0, 0};                      // own state (FP64)
    // window slots: own cell, then halo slots handled by the first 2*(TI+TJ) threads
    for (int slot = 0; slot < 2; slot++) {
        int wi, wj;   // window coordinates (0..WI-1, 0..WJ-1)
        bool act;
        if (slot == 0) {
            wi = li + 1; wj = lj + 1; act = own;
        } else {
            const int h = tid;
            // halo rows above/below the tile (columns 1..hi_j) and columns left/right (rows 1..hi_i)
            if (h < TJ) { wi = 0; wj = h + 1; act = h < hi_j && i0 > 0; }
            else if (h < 2 * TJ) { wi = hi_i + 1; wj = h - TJ + 1; act = h - TJ < hi_j && i0 + hi_i < D.nx; }
            else if (h < 2 * TJ + TI) { wi = h - 2 * TJ + 1; wj = 0; act = h - 2 * TJ < hi_i && j0 > 0; }
            else if (h < 2 * TJ + 2 * TI) { wi = h - 2 * TJ - TI + 1; wj = hi_j + 1; act = h - 2 * TJ - TI < hi_i && j0 + hi_j < D.ny; }
            else { wi = -1; wj = -1; act = false; }
        }
        float dfp[4] = {0, 0, 0, 0}, dfm[4] = {0, 0, 0, 0}, dhp[4] = {0, 0, 0, 0}, dhm[4] = {0, 0, 0, 0};
        if (act) {
            const int ci = i0 + wi - 1, cj = j0 + wj - 1;
            const long idx = base + (long)ci * D.ny + cj;
            double c[4];
            cell_correction(A, D, ci, cj, c);
            float d[4];
            for (int k = 0; k < 4; k++) {
                if (KAHAN) {
                    float h = static_cast<const float*>(hin)[k * P + idx], l = lin[k * P + idx];
                    if (c[k] != 0.0) {
                        const double v = ((double)h + (double)l) + c[k];
                        split2(v, h, l);
                    }
                    float dh, dl;
                    ff_sub(h, l, S.fr.Uh[k], S.fr.Ul[k], dh, dl);
                    d[k] = __fadd_rn(dh, dl);
                    if (slot == 0) { Uh[k] = h; Ul[k] = l; }
                } else {
                    const double U = static_cast<const double*>(hin)[k * P + idx] + c[k];
                    d[k] = (float)(U - S.fr.U[k]);
                    if (slot == 0) Ud[k] = U;
                }
            }
            dflux2(S.fr.cx, S.fr.cy, d, dfp, dfm, dhp, dhm);
        }
        if (wi >= 0) {
            const int w = wi * WJ + wj;
#pragma unroll
            for (int k = 0; k < 4; k++) {
                S.f[k][w] = dfp[k]; S.f[4 + k][w] = dfm[k]; S.f[8 + k][w] = dhp[k]; S.f[12 + k][w] = dhm[k];
            }
        }
    }
    __syncthreads();
    if (!own) return;
    // ---- interface terms and the update of the own cell ----
    const int w = (li + 1) * WJ + (lj + 1);
    const int wW = w - WJ, wE = w + WJ, wS = w - 1, wN = w + 1;
    Edge* exo = A.step & 1 ? A.ex[1] : A.ex[0];
    Edge* eyo = A.step & 1 ? A.ey[1] : A.ey[0];
    int bad = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float fp = S.f[k][w], fm = S.f[4 + k][w], hp = S.f[8 + k][w], hm = S.f[12 + k][w];
        float ah = 0.f, al = 0.f, th, tl;
        // x west
        if (i > 0) {
            const float Dw = __fadd_rn(S.f[k][wW], fm);
            lam_mul(lxh, lxl, Dw, th, tl);
            two_sum_acc(ah, al, th); al = __fadd_rn(al, tl);
            if (li == 0) exo[D.ex_base + (long)(i / TI - 1) * D.ny + j].s[1][k] = D.lamx * S.fr.Fx[k] + ((double)th + (double)tl);
        } else {
            two_sum_acc(ah, al, S.wc[0][k][0]); al = __fadd_rn(al, S.wc[0][k][1]);
            if (k == 1) { lam_mul(lxh, lxl, __fmul_rn(2.f, fm), th, tl); two_sum_acc(ah, al, th); al = __fadd_rn(al, tl); }
        }
        // x east
        if (i < D.nx - 1) {
            const float De = __fadd_rn(fp, S.f[4 + k][wE]);
            lam_mul(lxh, lxl, De, th, tl);
            two_sum_acc(ah, al, -th); al = __fadd_rn(al, -tl);
            if (li == hi_i - 1) exo[D.ex_base + (long)((i + 1) / TI - 1) * D.ny + j].s[0][k] = D.lamx * S.fr.Fx[k] + ((double)th + (double)tl);
        } else {
            two_sum_acc(ah, al, S.wc[1][k][0]); al = __fadd_rn(al, S.wc[1][k][1]);
            if (k == 1) { lam_mul(lxh, lxl, -__fmul_rn(2.f, fp), th, tl); two_sum_acc(ah, al, th); al = __fadd_rn(al, tl); }
        }
        // y south
        if (j > 0) {
            const float Ds = __fadd_rn(S.f[8 + k][wS], hm);
            lam_mul(lyh, lyl, Ds, th, tl);
            two_sum_acc(ah, al, th); al = __fadd_rn(al, tl);
            if (lj == 0) eyo[D.ey_base + (long)(j / TJ - 1) * D.nx + i].s[1][k] = D.lamy * S.fr.Fy[k] + ((double)th + (double)tl);
        } else {
            two_sum_acc(ah, al, S.wc[2][k][0]); al = __fadd_rn(al, S.wc[2][k][1]);
            if (k == 2) { lam_mul(lyh, lyl, __fmul_rn(2.f, hm), th, tl); two_sum_acc(ah, al, th); al = __fadd_rn(al, tl); }
        }
        // y north
        if (j < D.ny - 1) {
            const float Dn = __fadd_rn(hp, S.f[12 + k][wN]);
            lam_mul(lyh, lyl, Dn, th, tl);
            two_sum_acc(ah, al, -th); al = __fadd_rn(al, -tl);
            if (lj == hi_j - 1) eyo[D.ey_base + (long)((j + 1) / TJ - 1) * D.nx + i].s[0][k] = D.lamy * S.fr.Fy[k] + ((double)th + (double)tl);
        } else {
            two_sum_acc(ah, al, S.wc[3][k][0]); al = __fadd_rn(al, S.wc[3][k][1]);
            if (k == 2) { lam_mul(lyh, lyl, -__fmul_rn(2.f, hp), th, tl); two_sum_acc(ah, al, th); al = __fadd_rn(al, tl); }
        }
        const long idx = k * P + base + (long)i * D.ny + j;
        if (KAHAN) {
            float oh, ol;
            ff_add(Uh[k], Ul[k], ah, al, oh, ol);
            static_cast<float*>(hout)[idx] = oh;
            lout[idx] = ol;
            if (k == 0) bad |= !(oh > 0.f);
        } else {
            const double v = Ud[k] + ((double)ah + (double)al);
            static_cast<double*>(hout)[idx] = v;
            if (k == 0) bad |= !(v > 0.0);
        }
    }
    if (bad) {
        atomicOr(A.flag, SHLL_FLAG_NONPOSITIVE);
        atomicOr(&A.item_flags[tile.dom], SHLL_FLAG_NONPOSITIVE);
    }
}

// applies the last step's edge corrections to the edge cells (after the final step of a run)
template <bool KAHAN>
__global__ void k_fixup2d(Args2 A, int ndom) {
    const int d = blockIdx.y;
    if (d >= ndom) return;
    const Dom2 D = A.doms[d];
    if (D.steps <= 0) return;
    const long ncell = (long)D.nx * D.ny;
    const int buf = (D.par + D.steps) & 1;
    void* h = buf ? A.hi[1] : A.hi[0];
    float* l = buf ? A.lo[1] : A.lo[0];
    Args2 B = A;
    B.step = D.steps;  // corrections of step D.steps - 1
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (long)gridDim.x * blockDim.x) {
        const int i = (int)(c / D.ny), j = (int)(c % D.ny);
        if (!((i > 0 && i % TI == 0) || (j > 0 && j % TJ == 0))) continue;
        double corr[4];
        cell_correction(B, D, i, j, corr);
        for (int k = 0; k < 4; k++) {
            const long idx = k * A.plane + D.base + c;
            if (KAHAN) {
                float* hh = static_cast<float*>(h);
                const double v = ((double)hh[idx] + (double)l[idx]) + corr[k];
                split2(v, hh[idx], l[idx]);
            } else {
                static_cast<double*>(h)[idx] += corr[k];
            }
        }
    }
}

}  // namespace

// ------------------------------------------------------------------------------------------
struct Mixed2D {
    std::vector<Dom2> doms;
    std::vector<TileD> tiles;
    std::vector<int> par;
    long plane = 0, nex = 0, ney = 0;
    void* hi[2] = {nullptr, nullptr};
    float* lo[2] = {nullptr, nullptr};
    Edge* ex[2] = {nullptr, nullptr};
    Edge* ey[2] = {nullptr, nullptr};
    Dom2* d_doms = nullptr;
    TileD* d_tiles = nullptr;
};

static Mixed2D* get2(MixedState* m) { return static_cast<Mixed2D*>(*mixed_d2_slot(m)); }

MixedState* mixed2d_attach(MixedState* m, char* err, size_t len) {
    int count = 0;
    const shll_params* items = mixed_items(m, &count);
    for (int t = 0; t < count; t++) {
        if (items[t].order != 1) {
            snprintf(err, len, "2D mixed precision supports first order only (item %d)", t);
            return nullptr;
        }
    }
    Mixed2D* d = new Mixed2D();
    *mixed_d2_slot(m) = d;
    long off = 0, oex = 0, oey = 0;
    for (int t = 0; t < count; t++) {
        const shll_params& p = items[t];
        Dom2 D;
        memset(&D, 0, sizeof(D));
        D.base = off;
        D.nx = p.nx;
        D.ny = p.ny;
        D.tiles_i = (p.nx + TI - 1) / TI;
        D.tiles_j = (p.ny + TJ - 1) / TJ;
        D.ex_base = oex;
        D.ey_base = oey;
        D.gamma = p.gamma;
        D.R = p.R;
        D.CV = p.R / (p.gamma - 1.0);
        const double dx = p.lx / p.nx, dy = p.ly / p.ny;
        const double dt = (p.cfl / (p.R + 1)) * dx;
        D.lamx = p.cfl / (p.R + 1);
        D.lamy = dt / dy;
        d->doms.push_back(D);
        for (int a = 0; a < D.tiles_i; a++)
            for (int b = 0; b < D.tiles_j; b++) d->tiles.push_back({t, a, b});
        off += (long)p.nx * p.ny;
        oex += (long)(D.tiles_i - 1) * p.ny;
        oey += (long)(D.tiles_j - 1) * p.nx;
    }
    d->plane = off;
    d->nex = std::max(oex, 1L);
    d->ney = std::max(oey, 1L);
    d->par.assign(count, 0);
    const bool kahan = mixed_is_kahan(m);
    bool ok = true;
    for (int b = 0; b < 2 && ok; b++) {
        ok = cudaMalloc(&d->hi[b], (size_t)4 * off * (kahan ? sizeof(float) : sizeof(double))) == cudaSuccess;
        if (ok && kahan) ok = cudaMalloc(&d->lo[b], (size_t)4 * off * sizeof(float)) == cudaSuccess;
        if (ok) ok = cudaMalloc(&d->ex[b], sizeof(Edge) * d->nex) == cudaSuccess;
        if (ok) ok = cudaMalloc(&d->ey[b], sizeof(Edge) * d->ney) == cudaSuccess;
    }
    if (ok) ok = cudaMalloc(&d->d_doms, sizeof(Dom2) * count) == cudaSuccess;
    if (ok) ok = cudaMalloc(&d->d_tiles, sizeof(TileD) * d->tiles.size()) == cudaSuccess;
    if (ok) ok = cudaMemcpy(d->d_tiles, d->tiles.data(), sizeof(TileD) * d->tiles.size(), cudaMemcpyHostToDevice) == cudaSuccess;
    if (!ok) {
        snprintf(err, len, "2D mixed: device allocation failed (%ld cells)", off);
        mixed2d_detach(m);
        return nullptr;
    }
    return m;
}

void mixed2d_detach(MixedState* m) {
    Mixed2D* d = get2(m);
    if (!d) return;
    for (int b = 0; b < 2; b++) { cudaFree(d->hi[b]); cudaFree(d->lo[b]); cudaFree(d->ex[b]); cudaFree(d->ey[b]); }
    cudaFree(d->d_doms);
    cudaFree(d->d_tiles);
    delete d;
    *mixed_d2_slot(m) = nullptr;
}

// item's conserved state from primitive planes, U from P in FP64 (base_shll_2d.c:126-131)
int mixed2d_load(MixedState* m, int item, const double* prim, char* err, size_t len) {
    Mixed2D* d = get2(m);
    const Dom2& D = d->doms[item];
    const size_t n = (size_t)D.nx * D.ny;
    std::vector<double> U(4 * n);
    for (size_t c = 0; c < n; c++) {
        const double p0 = prim[c], p1 = prim[n + c], p2 = prim[2 * n + c], p3 = prim[3 * n + c];
        U[c] = p0;
        U[n + c] = p0 * p1;
        U[2 * n + c] = p0 * p2;
        U[3 * n + c] = p0 * (p3 * D.CV + 0.5 * (p1 * p1 + p2 * p2));
    }
    d->par[item] = 0;
    cudaStream_t s = mixed_stream(m);
    for (int k = 0; k < 4; k++) {
        const size_t off = (size_t)k * d->plane + D.base;
        cudaError_t e;
        if (mixed_is_kahan(m)) {
            std::vector<float> h(n), l(n);
            for (size_t c = 0; c < n; c++) {
                h[c] = (float)U[k * n + c];
                l[c] = (float)(U[k * n + c] - (double)h[c]);
            }
            e = cudaMemcpyAsync(static_cast<float*>(d->hi[0]) + off, h.data(), n * sizeof(float), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(d->lo[0] + off, l.data(), n * sizeof(float), cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        } else {
            e = cudaMemcpyAsync(static_cast<double*>(d->hi[0]) + off, U.data() + k * n, n * sizeof(double),
                                cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
        if (e != cudaSuccess) { snprintf(err, len, "2D state upload failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    }
    return SHLL_OK;
}

int mixed2d_run(MixedState* m, long nsteps, char* err, size_t len) {
    Mixed2D* d = get2(m);
    int count = 0;
    const shll_params* items = mixed_items(m, &count);
    long maxsteps = 0, updates = 0;
    for (int t = 0; t < count; t++) {
        const long s = nsteps >= 0 ? nsteps : shll_steps_for(&items[t]);
        d->doms[t].steps = (int)s;
        d->doms[t].par = d->par[t];
        maxsteps = std::max(maxsteps, s);
        updates += s * (long)d->doms[t].nx * d->doms[t].ny;
    }
    if (maxsteps == 0) return SHLL_OK;
    cudaStream_t s = mixed_stream(m);
    if (cudaMemcpyAsync(d->d_doms, d->doms.data(), sizeof(Dom2) * count, cudaMemcpyHostToDevice, s) != cudaSuccess) {
        snprintf(err, len, "2D descriptor upload failed");
        return SHLL_ERR_CUDA;
    }
    Args2 A;
    A.doms = d->d_doms;
    A.tiles = d->d_tiles;
    A.hi[0] = d->hi[0]; A.hi[1] = d->hi[1];
    A.lo[0] = d->lo[0]; A.lo[1] = d->lo[1];
    A.ex[0] = d->ex[0]; A.ex[1] = d->ex[1];
    A.ey[0] = d->ey[0]; A.ey[1] = d->ey[1];
    A.plane = d->plane;
    A.flag = mixed_flag_ptr(m);
    A.item_flags = mixed_item_flags_ptr(m);
    const bool kahan = mixed_is_kahan(m);
    const int ntiles = (int)d->tiles.size();
    shll_count_launches(maxsteps + 1);
    for (long st = 0; st < maxsteps; st++) {
        A.step = (int)st;
        if (kahan) k_step2d<true><<<ntiles, NT, 0, s>>>(A);
        else k_step2d<false><<<ntiles, NT, 0, s>>>(A);
    }
    dim3 fg(256, count);
    if (kahan) k_fixup2d<true><<<fg, 256, 0, s>>>(A, count);
    else k_fixup2d<false><<<fg, 256, 0, s>>>(A, count);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { snprintf(err, len, "2D step launch failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    for (int t = 0; t < count; t++) d->par[t] = (d->par[t] + d->doms[t].steps) & 1;
    mixed_add_updates(m, updates);
    return SHLL_OK;
}

int mixed2d_item_conserved(MixedState* m, int item, double* planes, char* err, size_t len) {
    Mixed2D* d = get2(m);
    const Dom2& D = d->doms[item];
    const size_t n = (size_t)D.nx * D.ny;
    const int b = d->par[item];
    cudaStream_t s = mixed_stream(m);
    for (int k = 0; k < 4; k++) {
        const size_t off = (size_t)k * d->plane + D.base;
        cudaError_t e;
        if (mixed_is_kahan(m)) {
            std::vector<float> h(n), l(n);
            e = cudaMemcpyAsync(h.data(), static_cast<float*>(d->hi[b]) + off, n * sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(l.data(), d->lo[b] + off, n * sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            for (size_t c = 0; c < n; c++) planes[k * n + c] = (double)h[c] + (double)l[c];
        } else {
            e = cudaMemcpyAsync(planes + k * n, static_cast<double*>(d->hi[b]) + off, n * sizeof(double),
                                cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        }
        if (e != cudaSuccess) { snprintf(err, len, "2D state download failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    }
    return SHLL_OK;
}

int mixed2d_totals(MixedState* m, int item, double* out, char* err, size_t len) {
    Mixed2D* d = get2(m);
    const Dom2& D = d->doms[item];
    const long n = (long)D.nx * D.ny;
    const int b = d->par[item];
    cudaStream_t s = mixed_stream(m);
    for (int k = 0; k < 4; k++) {
        const size_t off = (size_t)k * d->plane + D.base;
        cudaError_t e = mixed_is_kahan(m)
            ? device_pair_sums(static_cast<float*>(d->hi[b]) + off, d->lo[b] + off, 1, n, &out[k], s)
            : device_plane_sums(static_cast<double*>(d->hi[b]) + off, 64, 1, n, &out[k], s);
        if (e != cudaSuccess) { snprintf(err, len, "2D totals failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    }
    return SHLL_OK;
}

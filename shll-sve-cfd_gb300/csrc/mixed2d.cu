// Mixed-precision 2D SHLL engine (first order, reflective walls): FP32 split fluxes in
// perturbation form, state in FP64 (SHLL_PREC_MIXED_F64) or as an FP32 value + compensation pair
// (SHLL_PREC_MIXED_KAHAN); one launch per time step over every tile of every domain, with the
// stored state touched only once per fold window.
//
// The arithmetic is that of base-c/base_shll_2d.c:139-300 re-associated as interface fluxes:
// cell (i,j) gains lam_x (F_{i-1/2} - F_{i+1/2}) + lam_y (H_{j-1/2} - H_{j+1/2}), with
// F_{i+1/2} = fp_i + fm_{i+1} and the reflective walls of base_shll_2d.c:150-216 (x walls flip
// components 0,2,3 of the split flux, y walls 0,1,3, so the wall flux is (0, 2 fm1, 0, 0) at
// i = 0, (0, 2 fp1, 0, 0) at i = nx-1, (0, 0, 2 hm2, 0) at j = 0 and (0, 0, 2 hp2, 0) at j = ny-1).
//
//   * Fold windows of fold_steps steps.  At a fold (k_fold2d) the stored state B absorbs the
//     window's increments (FP64, or FP32-pair arithmetic), every tile (16 x 32 cells) gets a new
//     frame (the state of its centre cell and the split-flux coefficients derived from it, kept
//     in a per-tile table), and every cell stores C = B - U*(tile) rounded to FP32.
//   * Each step (k_step2d) evaluates the split fluxes of the tile's cells and of its one-cell halo in
//     FP32 as deviations from the tile's frame (own cells: C + P; halo cells: (B - U*) + P with the
//     neighbour's B in FP64), so rounding scales with |U - U*|; it sums the cell's four interface
//     terms exactly as an FP32 pair and adds them to the cell's increment pair P (TwoSum).
//   * Inside a tile both cells of an interface add the same FP32 term lam*Delta with opposite
//     signs.  Neighbouring tiles evaluate their shared interfaces in different frames; each tile
//     records the full flux it applied on its edges, and the east/north tile's edge cells then
//     receive lam*(F_west/south tile - F_own) (next step, or at the fold), so the west/south value
//     is the one that counts: mass, momentum and energy are conserved to the rounding of B.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
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
bool mixed_graph_replay_on(MixedState* m);
void mixed_set_tuning(MixedState* m, bool on);

namespace {

constexpr int TI = 16;           // tile rows (x, the slow index)
constexpr int TJ = 32;           // tile columns (y, contiguous)
constexpr int NT = TI * TJ;      // threads of the fold kernel, one cell each

// (the fields a step reads come first, in three aligned 16-byte groups, so that each thread loads
// them with three vector loads)
struct __align__(16) Dom2 {
    int base;                 // cell offset of the domain in the planes
    int nx, ny;
    int steps;                // steps of the current run
    int tiles_j;
    int tile_base;            // first tile of this domain in the tile / frame tables
    int ex_base, ey_base;     // first edge entry of this domain in the x / y edge buffers
    float lxh, lxl, lyh, lyl; // lam_x, lam_y as FP32 pairs
    int tiles_i;
    float alpha;              // MC limiter coefficient (second order, limiter 1)
    double gamma, R, CV, lamx, lamy;
};
static_assert(offsetof(Dom2, lxh) == 32 && offsetof(Dom2, tiles_i) == 48, "step fields in 16-byte groups");

struct __align__(16) TileD { int dom, ti, tj; };

// one edge interface: the full flux lam*F applied by the west/south tile (side 0) and by the
// east/north tile (side 1), four components each, as FP32 pairs (value, remainder)
struct __align__(16) Edge { float r[2][4][2]; };
static_assert(sizeof(Edge) == 64, "an edge record is four 16-byte vectors");

struct Frame2 {
    double U[4], Fx[4], Fy[4];
    double fmS1, fpS1, hmS2, hpS2;   // wall split fluxes (reflective walls)
    AnchorCoef cx, cy;               // coefficients for the x and y split fluxes
};

// anchor coefficients of a 2D tile frame, each duplicated into both FP32x2 lanes
struct Coef2D {
    float2 rho, u, v, nu, nv, ne, T, a, gR, R, cvinv, P, m, n, E, gm1;
    float2 Mx, nMx, Z1x, Z2x, My, nMy, Z1y, Z2y;
    float2 Fx[4], Fy[4], Uf[4];
};
__device__ __forceinline__ Coef2D coef2d(const AnchorCoef& cx, const AnchorCoef& cy) {
    Coef2D k;
    k.rho = f2(cx.rho); k.u = f2(cx.u); k.v = f2(cx.v); k.nu = f2(-cx.u); k.nv = f2(-cx.v); k.ne = f2(-cx.e);
    k.T = f2(cx.T); k.a = f2(cx.a); k.gR = f2(cx.gR); k.R = f2(cx.R); k.cvinv = f2(cx.cvinv); k.P = f2(cx.P);
    k.m = f2(cx.Uf[1]); k.n = f2(cx.Uf[2]); k.E = f2(cx.Uf[3]); k.gm1 = f2(__fmul_rn(cx.R, cx.cvinv));
    k.Mx = f2(cx.M); k.nMx = f2(-cx.M); k.Z1x = f2(cx.Z1); k.Z2x = f2(cx.Z2);
    k.My = f2(cy.M); k.nMy = f2(-cy.M); k.Z1y = f2(cy.Z1); k.Z2y = f2(cy.Z2);
    for (int q = 0; q < 4; q++) { k.Fx[q] = f2(cx.F[q]); k.Fy[q] = f2(cy.F[q]); k.Uf[q] = f2(cx.Uf[q]); }
    return k;
}

// What a step needs of its tile's frame, as FP32 values, pairs and FP32x2 coefficients (written
// once per fold window by k_tileconst2d, so that no step does FP64 arithmetic)
struct TileC2 {
    float wc[4][4][2];      // constant wall terms: [west, east, south, north][comp][pair]
    float lf[2][4][2];      // lam_x*Fx*, lam_y*Fy* of the frame as pairs
    float dn[4][4][2];      // U*(neighbour) - U*(this) as pairs: [west, east, south, north][comp]
    float dnd[4][4][2];     // the same for the diagonal neighbours: [(-1,-1), (-1,+1), (+1,-1), (+1,+1)]
    Coef2D cf;              // split-flux coefficients, duplicated into both lanes
};
constexpr int kTileC2Words = (int)(sizeof(TileC2) / 4);
static_assert(sizeof(TileC2) % 4 == 0, "word copy");

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



// dflux2 for two cells at once (same deviation identities, lane by lane; the minus fluxes from
// dfp + dfm = dF)
__device__ __forceinline__ void dflux2x2(const Coef2D& c, const float2 d[4], float2 fp[4], float2 fm[4],
                                         float2 hp[4], float2 hm[4]) {
    const float2 drho = d[0], dm = d[1], dn = d[2], dE = d[3];
    const float2 rho = add2(c.rho, drho);
    const float2 r = rcp2(rho);
    const float2 du = mul2(fma2(c.nu, drho, dm), r);
    const float2 dv = mul2(fma2(c.nv, drho, dn), r);
    const float2 u = add2(c.u, du), v = add2(c.v, dv);
    const float2 de = mul2(fma2(c.ne, drho, dE), r);
    const float2 ke = fma2(add2(u, c.u), du, mul2(add2(v, c.v), dv));  // d(u^2 + v^2)
    const float2 dT = mul2(fma2(f2(-0.5f), ke, de), c.cvinv);
    const float2 T = add2(c.T, dT);
    const float2 gRT = mul2(c.gR, T);
    const float2 ainv = rsqrt2(gRT);
    const float2 a = mul2(gRT, ainv);
    const float2 da = mul2(mul2(c.gR, dT), rcp2(add2(a, c.a)));
    // dP = (gamma-1)(dE - (dm u + m* du + dn v + n* dv) / 2): the energy form (see dflux1x2)
    const float2 dkin = fma2(dm, u, fma2(c.m, du, fma2(dn, v, mul2(c.n, dv))));
    const float2 dP = mul2(c.gm1, fma2(f2(-0.5f), dkin, dE));
    const float2 P = add2(c.P, dP);
    const float2 EP = add2(add2(c.E, dE), P), dEP = add2(dE, dP);
    {   // x direction, M = u / a
        const float2 dM = mul2(fma2(c.nMx, da, du), ainv);
        const float2 M = add2(c.Mx, dM);
        const float2 dZ1 = mul2(f2(0.5f), dM);
        const float2 Z1 = add2(c.Z1x, dZ1);
        const float2 dZ2 = mul2(f2(0.5f), fma2(da, fma2(neg2(M), M, f2(1.0f)), neg2(mul2(mul2(c.a, add2(M, c.Mx)), dM))));
        const float2 Z2 = add2(c.Z2x, dZ2);
        float2 dF[4];
        dF[0] = dm;
        dF[1] = add2(fma2(dm, u, mul2(c.m, du)), dP);
        dF[2] = fma2(dm, v, mul2(c.m, dv));
        dF[3] = fma2(du, EP, mul2(c.u, dEP));
#pragma unroll
        for (int k = 0; k < 4; k++) {
            fp[k] = add2(fma2(dF[k], Z1, mul2(c.Fx[k], dZ1)), fma2(d[k], Z2, mul2(c.Uf[k], dZ2)));
            fm[k] = sub2(dF[k], fp[k]);
        }
    }
    {   // y direction, M = v / a
        const float2 dM = mul2(fma2(c.nMy, da, dv), ainv);
        const float2 M = add2(c.My, dM);
        const float2 dZ1 = mul2(f2(0.5f), dM);
        const float2 Z1 = add2(c.Z1y, dZ1);
        const float2 dZ2 = mul2(f2(0.5f), fma2(da, fma2(neg2(M), M, f2(1.0f)), neg2(mul2(mul2(c.a, add2(M, c.My)), dM))));
        const float2 Z2 = add2(c.Z2y, dZ2);
        float2 dH[4];
        dH[0] = dn;
        dH[1] = fma2(dn, u, mul2(c.n, du));
        dH[2] = add2(fma2(dn, v, mul2(c.n, dv)), dP);
        dH[3] = fma2(dv, EP, mul2(c.v, dEP));
#pragma unroll
        for (int k = 0; k < 4; k++) {
            hp[k] = add2(fma2(dH[k], Z1, mul2(c.Fy[k], dZ1)), fma2(d[k], Z2, mul2(c.Uf[k], dZ2)));
            hm[k] = sub2(dH[k], hp[k]);
        }
    }
}

// Cell and plane offsets fit in 32 bits (the host refuses batches of more than 2^29 cells), so
// the kernels index with int: 64-bit integer multiply-adds would run on the slow FP64 pipe.
struct Args2 {
    const Dom2* doms;
    const TileD* tiles;
    Frame2* frames;      // per tile, written by the fold
    TileC2* tc;          // per tile, derived from the frames after each fold
    void* B;             // stored state: double[4][plane] or FP32 value planes (KAHAN)
    float* Blo;          // FP32 compensation planes (KAHAN)
    float* C;            // float[4][plane]: B - U*(tile) at the last fold
    // increment pairs since the last fold, by window step modulo 3, and the x / y edge records, by
    // step modulo 3: a launch of one or two steps reads the buffers of its first step and writes
    // those of its last + 1, never the ones it reads
    float* Ph[3];
    float* Pl[3];
    Edge* ex[3];
    Edge* ey[3];
    int plane;
    int step;            // global step of a k_step2d launch
    int s0, win;         // fold window: first step and length (k_fold2d)
    int* flag;
    int* item_flags;
};

// edge correction owed to cell (i, j) by the launch whose edge buffers have index pp (0..2):
// lam*(F of the west/south tile - F of the cell's own tile) on its west / south edge line, as an
// FP32 pair per component
// (each record is read as four 16-byte vectors: r[0][0..1], r[0][2..3], r[1][0..1], r[1][2..3])
__device__ __forceinline__ void add_edge(const Edge* e, float ch[4], float cl[4]) {
    const float4* v = reinterpret_cast<const float4*>(e);
    const float4 a0 = v[0], a1 = v[1], b0 = v[2], b1 = v[3];
    const float w[4][2] = {{a0.x, a0.y}, {a0.z, a0.w}, {a1.x, a1.y}, {a1.z, a1.w}};   // west/south tile
    const float o[4][2] = {{b0.x, b0.y}, {b0.z, b0.w}, {b1.x, b1.y}, {b1.z, b1.w}};   // own tile
#pragma unroll
    for (int k = 0; k < 4; k++) {
        two_sum_acc(ch[k], cl[k], w[k][0]);
        two_sum_acc(ch[k], cl[k], -o[k][0]);
        cl[k] = __fadd_rn(cl[k], __fadd_rn(w[k][1], -o[k][1]));
    }
}
__device__ __forceinline__ void edge_correction(const Args2& A, const Dom2& D, int i, int j, int pp, float ch[4],
                                                float cl[4]) {
    for (int k = 0; k < 4; k++) { ch[k] = 0.f; cl[k] = 0.f; }
    if (i > 0 && i % TI == 0) add_edge(&A.ex[pp][D.ex_base + (i / TI - 1) * D.ny + j], ch, cl);
    if (j > 0 && j % TJ == 0) add_edge(&A.ey[pp][D.ey_base + (j / TJ - 1) * D.nx + i], ch, cl);
}

__device__ __forceinline__ bool on_edge_line(int i, int j) { return (i > 0 && i % TI == 0) || (j > 0 && j % TJ == 0); }

// The increments so far (with the pending edge corrections of the previous step, pp) and C of the
// cell pair (i, jx), (i, jx + 1), with 8-byte loads: jx even and every domain of the batch with an
// even row length, so that the pair's index is even and the pair lies wholly inside or outside the
// domain (the caller checks inside).  Lane by lane the same arithmetic as the per-cell loads.
__device__ __forceinline__ void load_pair2(const Args2& A, const Dom2& D, int i, int jx, int kw, int pp,
                                           const float* phi, const float* pli, float2 h[4], float2 l[4],
                                           float2 c[4]) {
    const int cell = D.base + i * D.ny + jx;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int idx = k * A.plane + cell;
        h[k] = f2(0.f);
        l[k] = f2(0.f);
        if (kw > 0) {
            h[k] = *reinterpret_cast<const float2*>(phi + idx);
            l[k] = *reinterpret_cast<const float2*>(pli + idx);
        }
        c[k] = *reinterpret_cast<const float2*>(A.C + idx);
    }
    if (kw > 0) {
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (!on_edge_line(i, jx + q)) continue;
            float ch[4], cl[4];
            edge_correction(A, D, i, jx + q, pp, ch, cl);
#pragma unroll
            for (int k = 0; k < 4; k++) {   // the pending edge correction joins the increment pair
                float hh = lane(h[k], q), ll = lane(l[k], q);
                two_sum_acc(hh, ll, ch[k]);
                ll = __fadd_rn(ll, cl[k]);
                set_lane(h[k], q, hh);
                set_lane(l[k], q, ll);
            }
        }
    }
}

// ---- fold: B += P (+ the last edge corrections), new frames, C = B - U* ----
template <bool KAHAN>
__global__ void __launch_bounds__(NT) k_fold2d(Args2 A) {
    __shared__ double sU[4];
    __shared__ Frame2 fr;
    const TileD tile = A.tiles[blockIdx.x];
    const Dom2 D = A.doms[tile.dom];
    const int wd = min(max(D.steps - A.s0, 0), A.win);  // steps this domain took in the window
    if (A.win > 0 && wd == 0) return;                     // nothing changed since its last fold
    const int tid = threadIdx.x;
    const int i0 = tile.ti * TI, j0 = tile.tj * TJ;
    const int hi_i = min(TI, D.nx - i0), hi_j = min(TJ, D.ny - j0);
    const int li = tid / TJ, lj = tid % TJ;
    const int i = i0 + li, j = j0 + lj;
    const bool own = li < hi_i && lj < hi_j;
    const int P = A.plane;
    const int cell = D.base + i * D.ny + j;
    double U[4] = {0, 0, 0, 0};
    int bad = 0;
    if (own) {
        float ch[4] = {0, 0, 0, 0}, cl[4] = {0, 0, 0, 0};
        if (wd > 0 && on_edge_line(i, j)) edge_correction(A, D, i, j, (A.s0 + wd - 1) % 3, ch, cl);
        const float* ph = A.Ph[wd % 3];
        const float* pl = A.Pl[wd % 3];
        for (int k = 0; k < 4; k++) {
            const int idx = k * P + cell;
            if (KAHAN) {
                float h = static_cast<float*>(A.B)[idx], l = A.Blo[idx];
                if (wd > 0) {
                    float oh, ol, qh = ph[idx], ql = pl[idx];
                    two_sum_acc(qh, ql, ch[k]);
                    ql = __fadd_rn(ql, cl[k]);
                    ff_add(h, l, qh, ql, oh, ol);
                    h = oh; l = ol;
                    static_cast<float*>(A.B)[idx] = h;
                    A.Blo[idx] = l;
                }
                U[k] = (double)h + (double)l;
            } else {
                double v = static_cast<double*>(A.B)[idx];
                if (wd > 0) {
                    v = v + ((double)ph[idx] + (double)pl[idx]) + ((double)ch[k] + (double)cl[k]);
                    static_cast<double*>(A.B)[idx] = v;
                }
                U[k] = v;
            }
        }
        // breakdown: non-positive density or energy, or a non-finite state
        bad = !(U[0] > 0.0) || !(U[3] > 0.0) || !isfinite(U[0] + U[1] + U[2] + U[3]);
        if (li == hi_i / 2 && lj == hi_j / 2)
            for (int k = 0; k < 4; k++) sU[k] = U[k];
    }
    __syncthreads();
    if (tid == 0) {
        make_frame2(fr, sU, D);
        A.frames[D.tile_base + tile.ti * D.tiles_j + tile.tj] = fr;
    }
    __syncthreads();
    if (own)
        for (int k = 0; k < 4; k++) A.C[k * P + cell] = (float)(U[k] - fr.U[k]);
    if (bad) {
        atomicOr(A.flag, SHLL_FLAG_NONPOSITIVE);
        atomicOr(&A.item_flags[tile.dom], SHLL_FLAG_NONPOSITIVE);
    }
}

// ---- per-tile step constants of the new frames (after a fold) ----
__global__ void __launch_bounds__(64) k_tileconst2d(Args2 A) {
    const TileD tile = A.tiles[blockIdx.x];
    const Dom2 D = A.doms[tile.dom];
    const int wd = min(max(D.steps - A.s0, 0), A.win);
    if (A.win > 0 && wd == 0) return;   // frame unchanged
    const int tid = threadIdx.x;
    const int tb = D.tile_base + tile.ti * D.tiles_j + tile.tj;
    const Frame2& f = A.frames[tb];
    TileC2& c = A.tc[tb];
    if (tid == 16) c.cf = coef2d(f.cx, f.cy);
    if (tid < 16) {
        // constant wall terms: lam*(W_const - Fref) (west/south), lam*(Fref - W_const) (east/north)
        const int w = tid / 4, k = tid % 4;
        double v;
        if (w == 0) v = k == 1 ? D.lamx * (2.0 * f.fmS1 - f.Fx[1]) : -D.lamx * f.Fx[k];
        else if (w == 1) v = k == 1 ? D.lamx * (f.Fx[1] - 2.0 * f.fpS1) : D.lamx * f.Fx[k];
        else if (w == 2) v = k == 2 ? D.lamy * (2.0 * f.hmS2 - f.Fy[2]) : -D.lamy * f.Fy[k];
        else v = k == 2 ? D.lamy * (f.Fy[2] - 2.0 * f.hpS2) : D.lamy * f.Fy[k];
        split2(v, c.wc[w][k][0], c.wc[w][k][1]);
        if (tid < 8) {
            const int dir = tid / 4;
            split2(dir == 0 ? D.lamx * f.Fx[k] : D.lamy * f.Fy[k], c.lf[dir][k][0], c.lf[dir][k][1]);
        }
        // frame of the neighbour tile w (0 west = ti-1, 1 east, 2 south = tj-1, 3 north)
        const int ti = tile.ti + (w == 0 ? -1 : w == 1 ? 1 : 0), tj = tile.tj + (w == 2 ? -1 : w == 3 ? 1 : 0);
        double dU = 0.0;
        if (ti >= 0 && ti < D.tiles_i && tj >= 0 && tj < D.tiles_j)
            dU = A.frames[D.tile_base + ti * D.tiles_j + tj].U[k] - f.U[k];
        split2(dU, c.dn[w][k][0], c.dn[w][k][1]);
    } else if (tid >= 32 && tid < 48) {
        // the diagonal neighbour w: (ti -/+ 1, tj -/+ 1)
        const int w = (tid - 32) / 4, k = tid % 4;
        const int ti = tile.ti + (w < 2 ? -1 : 1), tj = tile.tj + ((w & 1) ? 1 : -1);
        double dU = 0.0;
        if (ti >= 0 && ti < D.tiles_i && tj >= 0 && tj < D.tiles_j)
            dU = A.frames[D.tile_base + ti * D.tiles_j + tj].U[k] - f.U[k];
        split2(dU, c.dnd[w][k][0], c.dnd[w][k][1]);
    }
}

// ---- one time step of one tile (packed: two cells per thread along j) ----
// 320 threads: threads 0..255 own the tile's 16 x 16 cell pairs (cells j, j+1 of a row); threads
// 256..319 evaluate the 64 halo pairs (the rows west and east of the tile, the column pairs south
// (j0-2, j0-1) and north (j0+32, j0+33)).  Every thread evaluates one pair's split fluxes, then,
// after the one barrier, each owner thread sums its pair's four interfaces per component.
constexpr int NTP = 320;
static_assert(kTileC2Words <= NTP, "the tile constants are copied one word per thread");
constexpr int WR = TI + 2;        // window rows (i0-1 .. i0+TI)
constexpr int WP = TJ / 2 + 2;    // window pairs per row (cells j0-2 .. j0+TJ+1)

struct Smem2 {
    float2 f[16][WR][WP];   // dfp0..3, dfm0..3, dhp0..3, dhm0..3 of the window pairs
    float wc[4][4][2];      // the tile's step constants (a copy of its TileC2)
    float lf[2][4][2];
    float dn[4][4][2];
    float dnd[4][4][2];
    Coef2D cf;
};

// VEC: every domain of the batch has an even row length; the pairs are loaded and stored with
// 8-byte accesses (load_pair2)
template <bool KAHAN, bool LAM_POW2, bool VEC>
__global__ void __launch_bounds__(NTP, 3) k_step2d(Args2 A) {
    __shared__ Smem2 S;
    const TileD tile = A.tiles[blockIdx.x];
    const Dom2 D = A.doms[tile.dom];
    if (A.step >= D.steps) return;
    const int tid = threadIdx.x;
    const int kw = A.step - A.s0;                       // step within the fold window
    const int i0 = tile.ti * TI, j0 = tile.tj * TJ;
    const int hi_i = min(TI, D.nx - i0), hi_j = min(TJ, D.ny - j0);
    const int P = A.plane;
    const int tb = D.tile_base + tile.ti * D.tiles_j + tile.tj;
    const float* phi = A.Ph[kw % 3];                     // increments so far (kw = 0: none)
    const float* pli = A.Pl[kw % 3];
    float* pho = A.Ph[(kw + 1) % 3];
    float* plo = A.Pl[(kw + 1) % 3];
    const int pp = (A.step + 2) % 3;                     // edge buffers of the previous step
    // the tile's step constants and coefficients, one word per thread into shared memory (read
    // from there after the barrier below, which keeps them out of the registers)
    if (tid < kTileC2Words)
        reinterpret_cast<float*>(&S.wc)[tid] = reinterpret_cast<const float*>(&A.tc[tb])[tid];

    // ---- this thread's window pair ----
    int r, c, nb;   // window row and pair column; owner tile of the cells (-1 this, 0 W, 1 E, 2 S, 3 N)
    bool act;
    if (tid < 256) {
        r = (tid >> 4) + 1; c = (tid & 15) + 1; nb = -1;
        act = r - 1 < hi_i && 2 * (c - 1) < hi_j;
    } else {
        const int h = tid - 256;
        if (h < 16) { r = 0; c = h + 1; nb = 0; act = i0 > 0 && 2 * h < hi_j; }
        else if (h < 32) { r = hi_i + 1; c = h - 15; nb = 1; act = i0 + hi_i < D.nx && 2 * (h - 16) < hi_j; }
        else if (h < 48) { r = h - 31; c = 0; nb = 2; act = j0 > 0 && h - 32 < hi_i; }
        else { r = h - 47; c = WP - 1; nb = 3; act = j0 + hi_j < D.ny && h - 48 < hi_i; }
    }
    const int ci = i0 + r - 1, cj = j0 + 2 * c - 2;     // cell of lane x; lane y is (ci, cj + 1)
    float2 Ph[4], Pl[4];                                 // own increment pairs
    __syncthreads();
    {
        float2 fp[4], fm[4], hp[4], hm[4];
        float2 d[4];
        for (int k = 0; k < 4; k++) { d[k] = f2(0.f); Ph[k] = f2(0.f); Pl[k] = f2(0.f); }
        if (act && VEC) {
            if (cj >= 0 && cj < D.ny) {                  // (outside the domain: zero deviation)
                float2 h2[4], l2[4], c2[4];
                load_pair2(A, D, ci, cj, kw, pp, phi, pli, h2, l2, c2);
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    if (nb < 0) { Ph[k] = h2[k]; Pl[k] = l2[k]; }
                    float2 base = c2[k];
                    if (nb >= 0) base = add2(add2(base, f2(S.dn[nb][k][0])), f2(S.dn[nb][k][1]));
                    d[k] = add2(base, add2(h2[k], l2[k]));
                }
            }
        } else if (act) {
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int cjq = cj + q;
                if (cjq < 0 || cjq >= D.ny) continue;    // outside the domain: zero deviation
                const int cell = D.base + ci * D.ny + cjq;
                float ch[4] = {0, 0, 0, 0}, cl[4] = {0, 0, 0, 0};
                const bool edge = kw > 0 && on_edge_line(ci, cjq);
                if (edge) edge_correction(A, D, ci, cjq, pp, ch, cl);
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int idx = k * P + cell;
                    float h = 0.f, l = 0.f;
                    if (kw > 0) { h = phi[idx]; l = pli[idx]; }
                    if (edge) {   // the pending edge correction joins the increment pair
                        two_sum_acc(h, l, ch[k]);
                        l = __fadd_rn(l, cl[k]);
                    }
                    if (nb < 0) { set_lane(Ph[k], q, h); set_lane(Pl[k], q, l); }
                    // deviation from this tile's frame: C (relative to the owner's frame) + the
                    // owner's frame offset + the increments
                    float base = A.C[idx];
                    if (nb >= 0) base = __fadd_rn(__fadd_rn(base, S.dn[nb][k][0]), S.dn[nb][k][1]);
                    set_lane(d[k], q, __fadd_rn(base, __fadd_rn(h, l)));
                }
            }
        }
        dflux2x2(S.cf, d, fp, fm, hp, hm);
        // every slot is written (inactive pairs with the frame's own zero deviations, so that a
        // masked-out neighbour read is finite), except that in a tile cut short in i the east halo
        // row coincides with the first unowned row: there the halo thread writes
        if (!(nb < 0 && r == hi_i + 1)) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                S.f[k][r][c] = fp[k]; S.f[4 + k][r][c] = fm[k]; S.f[8 + k][r][c] = hp[k]; S.f[12 + k][r][c] = hm[k];
            }
        }
    }
    __syncthreads();
    if (nb >= 0 || !act) return;

    // ---- interface terms and the increments of the own pair ----
    const int i = ci, jx = cj;                           // lane y: column jx + 1
    const bool has_y = jx + 1 < j0 + hi_j;
    const float2 lx2 = f2(D.lxh), lxl2 = f2(D.lxl), ly2 = f2(D.lyh), lyl2 = f2(D.lyl);
    // y walls: lane x at j = 0 (south), the lane at j = ny - 1 (north); their regular south / north
    // terms are masked and replaced by the wall terms below
    const bool wS = jx == 0, wNx = jx == D.ny - 1, wNy = has_y && jx + 1 == D.ny - 1;
    const float2 mS = make_float2(wS ? 0.f : 1.f, 1.f), mN = make_float2(wNx ? 0.f : 1.f, wNy ? 0.f : 1.f);
    Edge* exo = A.ex[A.step % 3];
    Edge* eyo = A.ey[A.step % 3];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float2 fp = S.f[k][r][c], fm = S.f[4 + k][r][c], hp = S.f[8 + k][r][c], hm = S.f[12 + k][r][c];
        float2 ah = Ph[k], al = Pl[k];
        auto lam = [&](float2 lh, float2 ll, float2 x, float2& th, float2& tl) {
            th = mul2(lh, x);
            tl = LAM_POW2 ? f2(0.f) : add2(fma2(lh, x, neg2(th)), mul2(ll, x));
        };
        auto acc = [&](float2 th, float2 tl) {   // (ah, al) += (th, tl)
            two_sum_acc2(ah, al, th);
            if (!LAM_POW2) al = add2(al, tl);
        };
        auto dec = [&](float2 th, float2 tl) {   // (ah, al) -= (th, tl)
            two_diff_acc2(ah, al, th);
            if (!LAM_POW2) al = sub2(al, tl);
        };
        float2 th, tl;
        // x west
        if (i > 0) {
            lam(lx2, lxl2, add2(S.f[k][r - 1][c], fm), th, tl);
            acc(th, tl);
            if (r == 1) {   // the tile's west edge: record the full flux this tile applied
                Edge* e = exo + D.ex_base + (i / TI - 1) * D.ny + jx;
                ff_add(S.lf[0][k][0], S.lf[0][k][1], th.x, tl.x, e[0].r[1][k][0], e[0].r[1][k][1]);
                if (has_y) ff_add(S.lf[0][k][0], S.lf[0][k][1], th.y, tl.y, e[1].r[1][k][0], e[1].r[1][k][1]);
            }
        } else {
            two_sum_acc2(ah, al, f2(S.wc[0][k][0]));   // wall constant: a full FP32 pair
            al = add2(al, f2(S.wc[0][k][1]));
            if (k == 1) { lam(lx2, lxl2, mul2(f2(2.f), fm), th, tl); acc(th, tl); }
        }
        // x east
        if (i < D.nx - 1) {
            lam(lx2, lxl2, add2(fp, S.f[4 + k][r + 1][c]), th, tl);
            dec(th, tl);
            if (r == hi_i) {
                Edge* e = exo + D.ex_base + ((i + 1) / TI - 1) * D.ny + jx;
                ff_add(S.lf[0][k][0], S.lf[0][k][1], th.x, tl.x, e[0].r[0][k][0], e[0].r[0][k][1]);
                if (has_y) ff_add(S.lf[0][k][0], S.lf[0][k][1], th.y, tl.y, e[1].r[0][k][0], e[1].r[0][k][1]);
            }
        } else {
            two_sum_acc2(ah, al, f2(S.wc[1][k][0]));
            al = add2(al, f2(S.wc[1][k][1]));
            if (k == 1) { lam(lx2, lxl2, mul2(f2(-2.f), fp), th, tl); acc(th, tl); }
        }
        // y south: lanes (jx-1 | jx) and (jx | jx+1)
        {
            const float hpS = S.f[8 + k][r][c - 1].y;
            lam(ly2, lyl2, add2(make_float2(hpS, hp.x), hm), th, tl);
            th = mul2(th, mS); tl = mul2(tl, mS);
            acc(th, tl);
            if (jx == j0 && j0 > 0) {   // the tile's south edge (lane x)
                float* rr = eyo[D.ey_base + (j0 / TJ - 1) * D.nx + i].r[1][k];
                ff_add(S.lf[1][k][0], S.lf[1][k][1], th.x, tl.x, rr[0], rr[1]);
            }
        }
        // y north: lanes (jx | jx+1) and (jx+1 | jx+2)
        {
            const float hmN = S.f[12 + k][r][c + 1].x;
            lam(ly2, lyl2, add2(hp, make_float2(hm.y, hmN)), th, tl);
            th = mul2(th, mN); tl = mul2(tl, mN);
            dec(th, tl);
            const int jn = j0 + hi_j - 1;   // the tile's north edge column
            if (jn + 1 < D.ny && (jx == jn || jx + 1 == jn)) {
                const int q = jx == jn ? 0 : 1;
                float* rr = eyo[D.ey_base + ((jn + 1) / TJ - 1) * D.nx + i].r[0][k];
                ff_add(S.lf[1][k][0], S.lf[1][k][1], lane(th, q), lane(tl, q), rr[0], rr[1]);
            }
        }
        // y walls
        if (wS || wNx || wNy) {
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const bool south = q == 0 && wS, north = q == 0 ? wNx : wNy;
                if (!south && !north) continue;
                float h = lane(ah, q), l = lane(al, q);
                const int w = south ? 2 : 3;
                two_sum_acc(h, l, S.wc[w][k][0]); l = __fadd_rn(l, S.wc[w][k][1]);
                if (k == 2) {   // +2 lam_y dhm2 (south), -2 lam_y dhp2 (north)
                    const float v = south ? __fmul_rn(2.f, lane(hm, q)) : __fmul_rn(-2.f, lane(hp, q));
                    const float vh = __fmul_rn(D.lyh, v);
                    const float vl = LAM_POW2 ? 0.f : __fadd_rn(__fmaf_rn(D.lyh, v, -vh), __fmul_rn(D.lyl, v));
                    two_sum_acc(h, l, vh); l = __fadd_rn(l, vl);
                }
                set_lane(ah, q, h); set_lane(al, q, l);
            }
        }
        const int cell = D.base + i * D.ny + jx;
        if (VEC) {   // (an even row length: both lanes are own cells)
            *reinterpret_cast<float2*>(pho + k * P + cell) = ah;
            *reinterpret_cast<float2*>(plo + k * P + cell) = al;
        } else {
            pho[k * P + cell] = ah.x;
            plo[k * P + cell] = al.x;
            if (has_y) {
                pho[k * P + cell + 1] = ah.y;
                plo[k * P + cell + 1] = al.y;
            }
        }
    }
}

// ---- two time steps of one tile per launch (temporal blocking) ----
// The tile's window is its 16 x 32 cells plus two cells on every side (20 rows x 18 pairs, the
// corners included, one thread per pair).  Step 1 evaluates the split fluxes of the whole window and
// updates every cell whose four neighbours are in it (the tile plus one cell around); step 2
// evaluates them again and updates the tile's own cells.  The increment pairs are loaded and stored
// once per two steps; the halo cells are updated in this tile's frame, as in the one-step kernel's
// halo evaluation.  The edge records are the sums of the two steps' applied fluxes, and the next
// launch applies the corrections as the one-step kernel does.  A domain with one step left takes one.
constexpr int NT2 = 384;                      // threads (20 x 18 = 360 window pairs)
constexpr int WR2 = TI + 4;                   // window rows i0-2 .. i0+TI+1
constexpr int kStep2Smem = 2 * 16 * WR2 * WP * (int)sizeof(float2);   // flux buffers of the two steps

struct Smem22 {
    float wc[4][4][2];      // the tile's step constants (a copy of its TileC2)
    float lf[2][4][2];
    float dn[4][4][2];
    float dnd[4][4][2];
    Coef2D cf;
    float recx[2][TJ][4][2];   // applied x fluxes summed over the steps: [west edge, east edge][column][comp]
    float recy[2][TI][4][2];   // applied y fluxes: [south edge, north edge][row][comp]
};
static_assert(sizeof(TileC2) == offsetof(Smem22, recx), "the tile constants are copied word for word");

template <bool KAHAN, bool LAM_POW2, bool VEC>
__global__ void __launch_bounds__(NT2, 2) k_step2d2(Args2 A) {
    __shared__ Smem22 S;
    extern __shared__ __align__(16) float2 g_flux2[];   // [step][16][WR2][WP]
    const TileD tile = A.tiles[blockIdx.x];
    const Dom2 D = A.doms[tile.dom];
    const int ns = min(2, D.steps - A.step);             // steps this domain takes in the launch
    if (ns <= 0) return;
    const int tid = threadIdx.x;
    const int kw = A.step - A.s0;                         // step within the fold window
    const int i0 = tile.ti * TI, j0 = tile.tj * TJ;
    const int hi_i = min(TI, D.nx - i0), hi_j = min(TJ, D.ny - j0);
    const int P = A.plane;
    const int tb = D.tile_base + tile.ti * D.tiles_j + tile.tj;
    const float* phi = A.Ph[kw % 3];                      // increments so far (kw = 0: none)
    const float* pli = A.Pl[kw % 3];
    float* pho = A.Ph[(kw + ns) % 3];
    float* plo = A.Pl[(kw + ns) % 3];
    const int pp = (A.step + 2) % 3;                      // edge buffers of the previous launch
    Edge* exo = A.ex[(A.step + ns - 1) % 3];
    Edge* eyo = A.ey[(A.step + ns - 1) % 3];
    if (tid < kTileC2Words)
        reinterpret_cast<float*>(&S.wc)[tid] = reinterpret_cast<const float*>(&A.tc[tb])[tid];
    auto flux = [&](int b, int q, int r, int c) -> float2& { return g_flux2[((b * 16 + q) * WR2 + r) * WP + c]; };

    // ---- this thread's window pair: row wr (cell row i), pair column wc (cells jx, jx + 1) ----
    const bool pt = tid < WR2 * WP;
    const int wr = pt ? tid / WP : 0, wc = pt ? tid % WP : 0;
    const int i = i0 - 2 + wr, jx = j0 - 2 + 2 * wc;
    bool ex[2];
#pragma unroll
    for (int q = 0; q < 2; q++) ex[q] = pt && i >= 0 && i < D.nx && jx + q >= 0 && jx + q < D.ny;
    // owner tile of the pair relative to this one (rows i0-2, i0-1 west, i0+16.. east; pair 0 south,
    // pair 17 north); -1: this tile
    const int di = wr < 2 ? -1 : (wr >= 2 + TI ? 1 : 0), dj = wc == 0 ? -1 : (wc == WP - 1 ? 1 : 0);
    const int nbi = di == 0 && dj == 0 ? -1
                  : dj == 0 ? (di < 0 ? 0 : 1)
                  : di == 0 ? (dj < 0 ? 2 : 3)
                  : 4 + (di < 0 ? 0 : 2) + (dj < 0 ? 0 : 1);
    // the update regions: step 1 the tile plus one cell around, step 2 (and the stores) the tile
    const bool r1 = wr >= 1 && wr <= TI + 2;
    const bool l1[2] = {ex[0] && r1 && jx >= j0 - 1 && jx <= j0 + TJ, ex[1] && r1 && jx + 1 >= j0 - 1 && jx + 1 <= j0 + TJ};
    const bool ro = wr >= 2 && wr < 2 + hi_i;
    const bool own[2] = {ex[0] && ro && jx >= j0 && jx < j0 + hi_j, ex[1] && ro && jx + 1 >= j0 && jx + 1 < j0 + hi_j};
    __syncthreads();   // (the tile constants)

    float2 base[4], ah[4], al[4];   // deviation of the pair at the launch's start, its increments
#pragma unroll
    for (int k = 0; k < 4; k++) { base[k] = f2(0.f); ah[k] = f2(0.f); al[k] = f2(0.f); }
    if (VEC && ex[0]) {   // (an even row length: the pair is inside or outside together)
        float2 c2[4];
        load_pair2(A, D, i, jx, kw, pp, phi, pli, ah, al, c2);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            base[k] = c2[k];
            if (nbi >= 0) {
                const float* o = nbi < 4 ? S.dn[nbi][k] : S.dnd[nbi - 4][k];
                base[k] = add2(add2(base[k], f2(o[0])), f2(o[1]));
            }
        }
    }
#pragma unroll
    for (int q = 0; q < 2 && !VEC; q++) {
        if (!ex[q]) continue;   // outside the domain: zero deviation (finite fluxes, never applied)
        const int cell = D.base + i * D.ny + jx + q;
        float ch[4] = {0, 0, 0, 0}, cl[4] = {0, 0, 0, 0};
        const bool edge = kw > 0 && on_edge_line(i, jx + q);
        if (edge) edge_correction(A, D, i, jx + q, pp, ch, cl);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int idx = k * P + cell;
            float h = 0.f, l = 0.f;
            if (kw > 0) { h = phi[idx]; l = pli[idx]; }
            if (edge) {   // the pending edge correction joins the increment pair
                two_sum_acc(h, l, ch[k]);
                l = __fadd_rn(l, cl[k]);
            }
            set_lane(ah[k], q, h);
            set_lane(al[k], q, l);
            // deviation from this tile's frame: C (relative to the owner's frame) + the owner's frame offset
            float b = A.C[idx];
            if (nbi >= 0) {
                const float* o = nbi < 4 ? S.dn[nbi][k] : S.dnd[nbi - 4][k];
                b = __fadd_rn(__fadd_rn(b, o[0]), o[1]);
            }
            set_lane(base[k], q, b);
        }
    }
    // edge records of the tile's own boundary cells (each written only by the cell's owner thread)
    const bool recW = ro && wr == 2 && i0 > 0, recE = ro && wr == 2 + hi_i - 1 && i + 1 < D.nx;
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (!own[q]) continue;
        const int col = jx + q - j0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (recW) { S.recx[0][col][k][0] = 0.f; S.recx[0][col][k][1] = 0.f; }
            if (recE) { S.recx[1][col][k][0] = 0.f; S.recx[1][col][k][1] = 0.f; }
            if (jx + q == j0 && j0 > 0) { S.recy[0][wr - 2][k][0] = 0.f; S.recy[0][wr - 2][k][1] = 0.f; }
            if (jx + q == j0 + hi_j - 1 && jx + q + 1 < D.ny) { S.recy[1][wr - 2][k][0] = 0.f; S.recy[1][wr - 2][k][1] = 0.f; }
        }
    }

    // split fluxes of the pair's current state into buffer b (every thread writes its slot)
    auto fluxes = [&](int b) {
        float2 d[4], fp[4], fm[4], hp[4], hm[4];
#pragma unroll
        for (int k = 0; k < 4; k++) d[k] = add2(base[k], add2(ah[k], al[k]));
        dflux2x2(S.cf, d, fp, fm, hp, hm);
        if (pt) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                flux(b, k, wr, wc) = fp[k]; flux(b, 4 + k, wr, wc) = fm[k];
                flux(b, 8 + k, wr, wc) = hp[k]; flux(b, 12 + k, wr, wc) = hm[k];
            }
        }
    };
    const float2 lx2 = f2(D.lxh), lxl2 = f2(D.lxl), ly2 = f2(D.lyh), lyl2 = f2(D.lyl);
    const bool wS = jx == 0, wNx = jx == D.ny - 1, wNy = jx + 1 == D.ny - 1;   // y walls per lane
    const float2 mS = make_float2(wS ? 0.f : 1.f, 1.f), mN = make_float2(wNx ? 0.f : 1.f, wNy ? 0.f : 1.f);
    const int cs = max(wc - 1, 0), cn = min(wc + 1, WP - 1);   // (clamped: the lanes they serve are masked)
    // one step's interface terms from buffer b added to the lanes `up`, the tile's edge records of the
    // lanes `rec` accumulated
    auto update = [&](int b, const bool up[2], const bool rec[2]) {
        auto lam = [&](float2 lh, float2 ll, float2 x, float2& th, float2& tl) {
            th = mul2(lh, x);
            tl = LAM_POW2 ? f2(0.f) : add2(fma2(lh, x, neg2(th)), mul2(ll, x));
        };
        auto record = [&](float* r, float th, float tl) { two_sum_acc(r[0], r[1], th); r[1] = __fadd_rn(r[1], tl); };
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float2 fp = flux(b, k, wr, wc), fm = flux(b, 4 + k, wr, wc);
            const float2 hp = flux(b, 8 + k, wr, wc), hm = flux(b, 12 + k, wr, wc);
            float2 h2 = ah[k], l2 = al[k];
            auto acc = [&](float2 th, float2 tl) {
                two_sum_acc2(h2, l2, th);
                if (!LAM_POW2) l2 = add2(l2, tl);
            };
            auto dec = [&](float2 th, float2 tl) {
                two_diff_acc2(h2, l2, th);
                if (!LAM_POW2) l2 = sub2(l2, tl);
            };
            float2 th, tl;
            // x west
            if (i > 0) {
                lam(lx2, lxl2, add2(flux(b, k, wr - 1, wc), fm), th, tl);
                acc(th, tl);
                if (recW)
                    for (int q = 0; q < 2; q++)
                        if (rec[q]) record(S.recx[0][jx + q - j0][k], lane(th, q), lane(tl, q));
            } else {
                two_sum_acc2(h2, l2, f2(S.wc[0][k][0]));
                l2 = add2(l2, f2(S.wc[0][k][1]));
                if (k == 1) { lam(lx2, lxl2, mul2(f2(2.f), fm), th, tl); acc(th, tl); }
            }
            // x east
            if (i < D.nx - 1) {
                lam(lx2, lxl2, add2(fp, flux(b, 4 + k, wr + 1, wc)), th, tl);
                dec(th, tl);
                if (recE)
                    for (int q = 0; q < 2; q++)
                        if (rec[q]) record(S.recx[1][jx + q - j0][k], lane(th, q), lane(tl, q));
            } else {
                two_sum_acc2(h2, l2, f2(S.wc[1][k][0]));
                l2 = add2(l2, f2(S.wc[1][k][1]));
                if (k == 1) { lam(lx2, lxl2, mul2(f2(-2.f), fp), th, tl); acc(th, tl); }
            }
            // y south: lanes (jx-1 | jx) and (jx | jx+1)
            {
                lam(ly2, lyl2, add2(make_float2(flux(b, 8 + k, wr, cs).y, hp.x), hm), th, tl);
                th = mul2(th, mS); tl = mul2(tl, mS);
                acc(th, tl);
                if (rec[0] && jx == j0 && j0 > 0) record(S.recy[0][wr - 2][k], th.x, tl.x);
            }
            // y north: lanes (jx | jx+1) and (jx+1 | jx+2)
            {
                lam(ly2, lyl2, add2(hp, make_float2(hm.y, flux(b, 12 + k, wr, cn).x)), th, tl);
                th = mul2(th, mN); tl = mul2(tl, mN);
                dec(th, tl);
                for (int q = 0; q < 2; q++)
                    if (rec[q] && jx + q == j0 + hi_j - 1 && jx + q + 1 < D.ny)
                        record(S.recy[1][wr - 2][k], lane(th, q), lane(tl, q));
            }
            // y walls
            if (wS || wNx || wNy) {
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const bool south = q == 0 && wS, north = q == 0 ? wNx : wNy;
                    if (!south && !north) continue;
                    float h = lane(h2, q), l = lane(l2, q);
                    const int w = south ? 2 : 3;
                    two_sum_acc(h, l, S.wc[w][k][0]); l = __fadd_rn(l, S.wc[w][k][1]);
                    if (k == 2) {   // +2 lam_y dhm2 (south), -2 lam_y dhp2 (north)
                        const float v = south ? __fmul_rn(2.f, lane(hm, q)) : __fmul_rn(-2.f, lane(hp, q));
                        const float vh = __fmul_rn(D.lyh, v);
                        const float vl = LAM_POW2 ? 0.f : __fadd_rn(__fmaf_rn(D.lyh, v, -vh), __fmul_rn(D.lyl, v));
                        two_sum_acc(h, l, vh); l = __fadd_rn(l, vl);
                    }
                    set_lane(h2, q, h); set_lane(l2, q, l);
                }
            }
            // only the lanes of the update region change
            ah[k] = make_float2(up[0] ? h2.x : ah[k].x, up[1] ? h2.y : ah[k].y);
            al[k] = make_float2(up[0] ? l2.x : al[k].x, up[1] ? l2.y : al[k].y);
        }
    };

    fluxes(0);
    __syncthreads();
    if (l1[0] || l1[1]) update(0, l1, own);
    if (ns == 2) {
        fluxes(1);
        __syncthreads();
        if (own[0] || own[1]) update(1, own, own);
    }

    // ---- the tile's increments and its edge records (full applied fluxes lam Fref ns + the sums) ----
    const float sc = (float)ns;   // (1 or 2: exact scaling of the pairs)
#pragma unroll
    for (int q = 0; q < 2; q++) {
        if (!own[q]) continue;
        const int cell = D.base + i * D.ny + jx + q;
        const int col = jx + q - j0;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (VEC) {   // (both lanes own: written once, from lane x)
                if (q == 0) {
                    *reinterpret_cast<float2*>(pho + k * P + cell) = ah[k];
                    *reinterpret_cast<float2*>(plo + k * P + cell) = al[k];
                }
            } else {
                pho[k * P + cell] = lane(ah[k], q);
                plo[k * P + cell] = lane(al[k], q);
            }
            const float lxh = __fmul_rn(sc, S.lf[0][k][0]), lxl = __fmul_rn(sc, S.lf[0][k][1]);
            const float lyh = __fmul_rn(sc, S.lf[1][k][0]), lyl = __fmul_rn(sc, S.lf[1][k][1]);
            if (recW) {
                float* rr = exo[D.ex_base + (i / TI - 1) * D.ny + jx + q].r[1][k];
                ff_add(lxh, lxl, S.recx[0][col][k][0], S.recx[0][col][k][1], rr[0], rr[1]);
            }
            if (recE) {
                float* rr = exo[D.ex_base + ((i + 1) / TI - 1) * D.ny + jx + q].r[0][k];
                ff_add(lxh, lxl, S.recx[1][col][k][0], S.recx[1][col][k][1], rr[0], rr[1]);
            }
            if (jx + q == j0 && j0 > 0) {
                float* rr = eyo[D.ey_base + (j0 / TJ - 1) * D.nx + i].r[1][k];
                ff_add(lyh, lyl, S.recy[0][wr - 2][k][0], S.recy[0][wr - 2][k][1], rr[0], rr[1]);
            }
            if (jx + q == j0 + hi_j - 1 && jx + q + 1 < D.ny) {
                float* rr = eyo[D.ey_base + ((jx + q + 1) / TJ - 1) * D.nx + i].r[0][k];
                ff_add(lyh, lyl, S.recy[1][wr - 2][k][0], S.recy[1][wr - 2][k][1], rr[0], rr[1]);
            }
        }
    }
}

// ---- one second-order time step of one tile ----
// The x and y sweeps of base-c/2nd_order_base_shll.c:203-459 (and the MC limiter of
// base-omp/2nd_order_base_shll.c:316-325) as interface fluxes: with the face values
// Lx_i = fp_i + sp_i/2 and Rx_i = fm_i - sm_i/2 (sp, sm the limited slopes of the split fluxes,
// zero on the domain's edge cells), F_{i+1/2} = Lx_i + Rx_{i+1}, and the cell gains
// lam_x (F_{i-1/2} - F_{i+1/2}) + lam_y (H_{j-1/2} - H_{j+1/2}).  At an outflow wall the wall flux is
// the wall cell's own Lx + Rx = fp + fm (2nd_order_base_shll.c:236-262), so the frame's reference
// flux cancels from every increment and the walls need no constant terms.
// The window is the tile and two cells on each side (20 rows x 18 pairs; the corner pairs are not
// needed), one thread per pair.  Phase 1: split-flux deviations of every window pair in this
// tile's frame.  Phase 2: face values, x for the rows i0-1 .. i0+16 of the tile's columns, y for the
// tile's rows and the columns j0-1 .. j0+32.  Phase 3: the own pairs' four interfaces, TwoSum into
// their increment pairs, and the tile's edge records (as in the first-order kernel).
constexpr int kStepO2Smem = 2 * 16 * WR2 * WP * (int)sizeof(float2);   // split fluxes, face values

struct SmemO2 {             // the tile's step constants (a copy of its TileC2)
    float wc[4][4][2];
    float lf[2][4][2];
    float dn[4][4][2];
    float dnd[4][4][2];
    Coef2D cf;
};
static_assert(sizeof(SmemO2) == sizeof(TileC2), "the tile constants are copied word for word");

template <bool KAHAN, bool LAM_POW2, int LIM, bool VEC>
__global__ void __launch_bounds__(NT2, 2) k_step2d_o2(Args2 A) {
    __shared__ SmemO2 S;
    extern __shared__ __align__(16) float2 g_o2[];   // [32][WR2][WP]: fp fm hp hm, then Lx Rx Ly Ry
    const TileD tile = A.tiles[blockIdx.x];
    const Dom2 D = A.doms[tile.dom];
    if (A.step >= D.steps) return;
    const int tid = threadIdx.x;
    const int kw = A.step - A.s0;                         // step within the fold window
    const int i0 = tile.ti * TI, j0 = tile.tj * TJ;
    const int hi_i = min(TI, D.nx - i0), hi_j = min(TJ, D.ny - j0);
    const int P = A.plane;
    const int tb = D.tile_base + tile.ti * D.tiles_j + tile.tj;
    const float* phi = A.Ph[kw % 3];                      // increments so far (kw = 0: none)
    const float* pli = A.Pl[kw % 3];
    float* pho = A.Ph[(kw + 1) % 3];
    float* plo = A.Pl[(kw + 1) % 3];
    const int pp = (A.step + 2) % 3;                      // edge buffers of the previous step
    if (tid < kTileC2Words)
        reinterpret_cast<float*>(&S)[tid] = reinterpret_cast<const float*>(&A.tc[tb])[tid];
    auto fl = [&](int q, int r, int c) -> float2& { return g_o2[(q * WR2 + r) * WP + c]; };

    // ---- this thread's window pair: row wr (cell row i), pair column wc (cells jx, jx + 1) ----
    const bool pt = tid < WR2 * WP;
    const int wr = pt ? tid / WP : 0, wc = pt ? tid % WP : 0;
    const int i = i0 - 2 + wr, jx = j0 - 2 + 2 * wc;
    const int di = wr < 2 ? -1 : (wr >= 2 + TI ? 1 : 0), dj = wc == 0 ? -1 : (wc == WP - 1 ? 1 : 0);
    // owner tile of the pair (-1 this tile, 0 W, 1 E, 2 S, 3 N); corner pairs are left out
    const int nbi = di == 0 && dj == 0 ? -1 : dj == 0 ? (di < 0 ? 0 : 1) : (dj < 0 ? 2 : 3);
    bool ex[2];
#pragma unroll
    for (int q = 0; q < 2; q++)
        ex[q] = pt && (di == 0 || dj == 0) && i >= 0 && i < D.nx && jx + q >= 0 && jx + q < D.ny;
    const bool ro = wr >= 2 && wr < 2 + hi_i;
    const bool own[2] = {ex[0] && ro && jx >= j0 && jx < j0 + hi_j, ex[1] && ro && jx + 1 >= j0 && jx + 1 < j0 + hi_j};
    __syncthreads();   // (the tile constants)

    // ---- phase 1: deviations and split fluxes ----
    float2 ah[4], al[4];   // the pair's increments so far (own pairs)
    {
        float2 d[4];
#pragma unroll
        for (int k = 0; k < 4; k++) { d[k] = f2(0.f); ah[k] = f2(0.f); al[k] = f2(0.f); }
        if (VEC && ex[0]) {   // (an even row length: the pair is inside or outside together)
            float2 c2[4];
            load_pair2(A, D, i, jx, kw, pp, phi, pli, ah, al, c2);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                float2 b = c2[k];
                if (nbi >= 0) b = add2(add2(b, f2(S.dn[nbi][k][0])), f2(S.dn[nbi][k][1]));
                d[k] = add2(b, add2(ah[k], al[k]));
            }
        }
#pragma unroll
        for (int q = 0; q < 2 && !VEC; q++) {
            if (!ex[q]) continue;   // outside the domain or a corner: zero deviation (finite, never applied)
            const int cell = D.base + i * D.ny + jx + q;
            float ch[4] = {0, 0, 0, 0}, cl[4] = {0, 0, 0, 0};
            const bool edge = kw > 0 && on_edge_line(i, jx + q);
            if (edge) edge_correction(A, D, i, jx + q, pp, ch, cl);
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const int idx = k * P + cell;
                float h = 0.f, l = 0.f;
                if (kw > 0) { h = phi[idx]; l = pli[idx]; }
                if (edge) {   // the pending edge correction joins the increment pair
                    two_sum_acc(h, l, ch[k]);
                    l = __fadd_rn(l, cl[k]);
                }
                set_lane(ah[k], q, h);
                set_lane(al[k], q, l);
                float b = A.C[idx];
                if (nbi >= 0) b = __fadd_rn(__fadd_rn(b, S.dn[nbi][k][0]), S.dn[nbi][k][1]);
                set_lane(d[k], q, __fadd_rn(b, __fadd_rn(h, l)));
            }
        }
        float2 fp[4], fm[4], hp[4], hm[4];
        dflux2x2(S.cf, d, fp, fm, hp, hm);
        if (pt) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                fl(k, wr, wc) = fp[k]; fl(4 + k, wr, wc) = fm[k];
                fl(8 + k, wr, wc) = hp[k]; fl(12 + k, wr, wc) = hm[k];
            }
        }
    }
    __syncthreads();

    // ---- phase 2: face values ----
    const float alpha = D.alpha;
    if (pt && wr >= 1 && wr <= TI + 2 && wc >= 1 && wc <= TJ / 2) {
        // x: slopes along i, zero on the edge cells i = 0, nx - 1 (and outside the domain)
        const float hx = (i <= 0 || i >= D.nx - 1) ? 0.f : 0.5f;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float2 pm = fl(k, wr - 1, wc), pc = fl(k, wr, wc), pq = fl(k, wr + 1, wc);
            fl(16 + k, wr, wc) = fma2(f2(hx), slope2<LIM>(sub2(pc, pm), sub2(pq, pc), alpha), pc);
            const float2 mm = fl(4 + k, wr - 1, wc), mc = fl(4 + k, wr, wc), mq = fl(4 + k, wr + 1, wc);
            fl(20 + k, wr, wc) = fma2(f2(-hx), slope2<LIM>(sub2(mc, mm), sub2(mq, mc), alpha), mc);
        }
    }
    if (pt && wr >= 2 && wr < 2 + TI) {
        // y: slopes along j (lane x needs the south pair's lane y, lane y the north pair's lane x;
        // the clamped neighbours only serve lanes that no interface reads), zero on j = 0, ny - 1
        const int cs = max(wc - 1, 0), cn = min(wc + 1, WP - 1);
        const float2 hy = make_float2((jx <= 0 || jx >= D.ny - 1) ? 0.f : 0.5f,
                                      (jx + 1 <= 0 || jx + 1 >= D.ny - 1) ? 0.f : 0.5f);
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const float2 pc = fl(8 + k, wr, wc);
            const float2 pb = make_float2(fl(8 + k, wr, cs).y, pc.x), pn = make_float2(pc.y, fl(8 + k, wr, cn).x);
            fl(24 + k, wr, wc) = fma2(hy, slope2<LIM>(sub2(pc, pb), sub2(pn, pc), alpha), pc);
            const float2 mc = fl(12 + k, wr, wc);
            const float2 mb = make_float2(fl(12 + k, wr, cs).y, mc.x), mn = make_float2(mc.y, fl(12 + k, wr, cn).x);
            fl(28 + k, wr, wc) = fma2(neg2(hy), slope2<LIM>(sub2(mc, mb), sub2(mn, mc), alpha), mc);
        }
    }
    __syncthreads();
    if (!(own[0] || own[1])) return;

    // ---- phase 3: interfaces and increments of the own pair ----
    const bool has_y = own[1];
    const float2 lx2 = f2(D.lxh), lxl2 = f2(D.lxl), ly2 = f2(D.lyh), lyl2 = f2(D.lyl);
    const bool wW = i == 0, wE = i == D.nx - 1;                       // x walls (whole pair)
    const bool wS = jx == 0, wNx = jx == D.ny - 1, wNy = jx + 1 == D.ny - 1;   // y walls per lane
    const bool recW = wr == 2 && i0 > 0, recE = wr == 2 + hi_i - 1 && i + 1 < D.nx;
    const int jn = j0 + hi_j - 1;   // the tile's north edge column
    const bool recN = jn + 1 < D.ny && (jx == jn || jx + 1 == jn);
    const int qn = jx == jn ? 0 : 1;
    Edge* exo = A.ex[A.step % 3];
    Edge* eyo = A.ey[A.step % 3];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float2 Lx = fl(16 + k, wr, wc), Rx = fl(20 + k, wr, wc);
        const float2 Ly = fl(24 + k, wr, wc), Ry = fl(28 + k, wr, wc);
        float2 h = ah[k], l = al[k];
        auto lam = [&](float2 lh, float2 ll, float2 x, float2& th, float2& tl) {
            th = mul2(lh, x);
            tl = LAM_POW2 ? f2(0.f) : add2(fma2(lh, x, neg2(th)), mul2(ll, x));
        };
        float2 th, tl;
        // x west: F_{i-1/2} = Lx_{i-1} + Rx_i (wall: the cell's own Lx + Rx)
        lam(lx2, lxl2, add2(wW ? Lx : fl(16 + k, wr - 1, wc), Rx), th, tl);
        two_sum_acc2(h, l, th);
        if (!LAM_POW2) l = add2(l, tl);
        if (recW) {   // the tile's west edge: record the full flux this tile applied
            Edge* e = exo + D.ex_base + (i / TI - 1) * D.ny + jx;
            ff_add(S.lf[0][k][0], S.lf[0][k][1], th.x, tl.x, e[0].r[1][k][0], e[0].r[1][k][1]);
            if (has_y) ff_add(S.lf[0][k][0], S.lf[0][k][1], th.y, tl.y, e[1].r[1][k][0], e[1].r[1][k][1]);
        }
        // x east: F_{i+1/2} = Lx_i + Rx_{i+1}
        lam(lx2, lxl2, add2(Lx, wE ? Rx : fl(20 + k, wr + 1, wc)), th, tl);
        two_diff_acc2(h, l, th);
        if (!LAM_POW2) l = sub2(l, tl);
        if (recE) {
            Edge* e = exo + D.ex_base + ((i + 1) / TI - 1) * D.ny + jx;
            ff_add(S.lf[0][k][0], S.lf[0][k][1], th.x, tl.x, e[0].r[0][k][0], e[0].r[0][k][1]);
            if (has_y) ff_add(S.lf[0][k][0], S.lf[0][k][1], th.y, tl.y, e[1].r[0][k][0], e[1].r[0][k][1]);
        }
        // y south: lanes (jx-1 | jx) and (jx | jx+1); lane x at the south wall: its own Ly + Ry
        lam(ly2, lyl2, add2(make_float2(wS ? Ly.x : fl(24 + k, wr, wc - 1).y, Ly.x), Ry), th, tl);
        two_sum_acc2(h, l, th);
        if (!LAM_POW2) l = add2(l, tl);
        if (jx == j0 && j0 > 0) {   // the tile's south edge (lane x)
            float* rr = eyo[D.ey_base + (j0 / TJ - 1) * D.nx + i].r[1][k];
            ff_add(S.lf[1][k][0], S.lf[1][k][1], th.x, tl.x, rr[0], rr[1]);
        }
        // y north: lanes (jx | jx+1) and (jx+1 | jx+2); at the north wall the lane's own Ly + Ry
        lam(ly2, lyl2, add2(Ly, make_float2(wNx ? Ry.x : Ry.y, wNy ? Ry.y : fl(28 + k, wr, min(wc + 1, WP - 1)).x)), th, tl);
        two_diff_acc2(h, l, th);
        if (!LAM_POW2) l = sub2(l, tl);
        if (recN) {
            float* rr = eyo[D.ey_base + ((jn + 1) / TJ - 1) * D.nx + i].r[0][k];
            ff_add(S.lf[1][k][0], S.lf[1][k][1], lane(th, qn), lane(tl, qn), rr[0], rr[1]);
        }
        const int cell = D.base + i * D.ny + jx;
        if (VEC) {   // (both lanes own)
            *reinterpret_cast<float2*>(pho + k * P + cell) = h;
            *reinterpret_cast<float2*>(plo + k * P + cell) = l;
        } else {
            if (own[0]) { pho[k * P + cell] = h.x; plo[k * P + cell] = l.x; }
            if (has_y) { pho[k * P + cell + 1] = h.y; plo[k * P + cell + 1] = l.y; }
        }
    }
}

}  // namespace

// ------------------------------------------------------------------------------------------
// steps per step launch of a new 2D state until the tuner chooses (SHLL_2D_STEPS_PER_LAUNCH = 1 or 2
// overrides the library's default, 2)
static int default_kstep() {
    const char* v = getenv("SHLL_2D_STEPS_PER_LAUNCH");
    return v && v[0] == '1' ? 1 : 2;
}

struct Mixed2D {
    std::vector<Dom2> doms;
    std::vector<TileD> tiles;
    long plane = 0, nex = 0, ney = 0;
    void* B = nullptr;
    float* Blo = nullptr;
    float* C = nullptr;
    float* Ph[3] = {nullptr, nullptr, nullptr};
    float* Pl[3] = {nullptr, nullptr, nullptr};
    Edge* ex[3] = {nullptr, nullptr, nullptr};
    Edge* ey[3] = {nullptr, nullptr, nullptr};
    Frame2* frames = nullptr;
    TileC2* tc = nullptr;
    Dom2* d_doms = nullptr;
    TileD* d_tiles = nullptr;
    int fold = 16;
    int order = 1, lim = 0;        // the batch's scheme (second order: minmod 0 or MC 1)
    bool vec = false;              // every domain has an even row length (8-byte pair accesses)
    int kstep = default_kstep();   // time steps per step launch (k_step2d2 for 2, k_step2d for 1)
    // device checkpoint of the stored state (a run starts with a fold that rebuilds frames, C and
    // the tile constants from it, so the stored state is the whole state between runs)
    void* ckB = nullptr;
    float* ckBlo = nullptr;
    // captured launch sequences of earlier runs (per-domain step counts and fold window), replayed
    // when a run repeats
    struct GraphEntry { std::vector<int> steps; int fold, kstep; cudaGraphExec_t exec; long launches; };
    std::vector<GraphEntry> graphs;
    std::vector<std::pair<std::vector<int>, int>> seen;   // (step counts, fold * 4 + kstep)
};

// fold windows chosen by the autotuner, process-wide, by (state format and scheme, floor(log2 of the
// largest domain's cells)); applied to later 2D batches whose items leave fold_steps at 0
static std::mutex g_tune2d_mu;
static std::map<std::pair<int, int>, std::pair<int, int>> g_tune2d;   // -> (fold window, steps per launch)

static std::pair<int, int> tune2d_key(const std::vector<Dom2>& doms, bool kahan, int order, int lim) {
    long cells = 1;
    for (const Dom2& D : doms) cells = std::max(cells, (long)D.nx * D.ny);
    int lg = 0;
    while ((2L << lg) <= cells) lg++;
    return {(kahan ? 1 : 0) + 2 * (order == 2 ? 1 + lim : 0), lg};
}

static Mixed2D* get2(MixedState* m) { return static_cast<Mixed2D*>(*mixed_d2_slot(m)); }
int mixed_fold(MixedState* m);

MixedState* mixed2d_attach(MixedState* m, char* err, size_t len) {
    int count = 0;
    const shll_params* items = mixed_items(m, &count);
    for (int t = 0; t < count; t++) {
        // one scheme per batch: the step kernel is specialised on the order and the limiter
        if (items[t].order != items[0].order || (items[0].order == 2 && items[t].limiter != items[0].limiter)) {
            snprintf(err, len, "2D mixed precision: every domain of a batch needs the same order and limiter (item %d)", t);
            return nullptr;
        }
    }
    Mixed2D* d = new Mixed2D();
    *mixed_d2_slot(m) = d;
    d->order = items[0].order;
    d->lim = d->order == 2 && items[0].limiter == 1 ? 1 : 0;
    if (d->order == 2) d->kstep = 1;   // (the two-step kernel is first order)
    d->fold = std::max(1, mixed_fold(m));
    long off = 0, oex = 0, oey = 0, otile = 0;
    for (int t = 0; t < count; t++) {
        const shll_params& p = items[t];
        Dom2 D;
        memset(&D, 0, sizeof(D));
        D.base = (int)off;
        D.nx = p.nx;
        D.ny = p.ny;
        D.tiles_i = (p.nx + TI - 1) / TI;
        D.tiles_j = (p.ny + TJ - 1) / TJ;
        D.tile_base = (int)otile;
        D.ex_base = (int)oex;
        D.ey_base = (int)oey;
        D.gamma = p.gamma;
        D.R = p.R;
        D.CV = p.R / (p.gamma - 1.0);
        const double dx = p.lx / p.nx, dy = p.ly / p.ny;
        const double dt = (p.cfl / (p.R + 1)) * dx;
        D.lamx = p.cfl / (p.R + 1);
        D.lamy = dt / dy;
        D.lxh = (float)D.lamx; D.lxl = (float)(D.lamx - (double)D.lxh);
        D.lyh = (float)D.lamy; D.lyl = (float)(D.lamy - (double)D.lyh);
        D.alpha = (float)p.mc_alpha;
        d->doms.push_back(D);
        for (int a = 0; a < D.tiles_i; a++)
            for (int b = 0; b < D.tiles_j; b++) d->tiles.push_back({t, a, b});
        off += (long)p.nx * p.ny;
        otile += (long)D.tiles_i * D.tiles_j;
        oex += (long)(D.tiles_i - 1) * p.ny;
        oey += (long)(D.tiles_j - 1) * p.nx;
    }
    if (4 * off >= (1L << 31) || oex >= (1L << 31) || oey >= (1L << 31)) {
        snprintf(err, len, "2D mixed: %ld cells exceed the 2^29-cell limit of a batch", off);
        delete d;
        *mixed_d2_slot(m) = nullptr;
        return nullptr;
    }
    if (items[0].fold_steps <= 0) {   // a tuned fold window of this class
        std::lock_guard<std::mutex> lk(g_tune2d_mu);
        auto it = g_tune2d.find(tune2d_key(d->doms, mixed_is_kahan(m), d->order, d->lim));
        if (it != g_tune2d.end()) { d->fold = it->second.first; if (d->order == 1) d->kstep = it->second.second; }
    }
    d->plane = off;
    // (SHLL_2D_SCALAR_PAIRS set: per-cell accesses everywhere, the same results)
    d->vec = std::getenv("SHLL_2D_SCALAR_PAIRS") == nullptr;
    for (const Dom2& D : d->doms) d->vec = d->vec && D.ny % 2 == 0;
    d->nex = std::max(oex, 1L);
    d->ney = std::max(oey, 1L);
    const bool kahan = mixed_is_kahan(m);
    const size_t nf = (size_t)4 * off;
    bool ok = cudaMalloc(&d->B, nf * (kahan ? sizeof(float) : sizeof(double))) == cudaSuccess;
    if (ok && kahan) ok = cudaMalloc(&d->Blo, nf * sizeof(float)) == cudaSuccess;
    if (ok) ok = cudaMalloc(&d->C, nf * sizeof(float)) == cudaSuccess;
    for (int b = 0; b < 3 && ok; b++) {
        ok = cudaMalloc(&d->Ph[b], nf * sizeof(float)) == cudaSuccess;
        if (ok) ok = cudaMalloc(&d->Pl[b], nf * sizeof(float)) == cudaSuccess;
        if (ok) ok = cudaMalloc(&d->ex[b], sizeof(Edge) * d->nex) == cudaSuccess;
        if (ok) ok = cudaMalloc(&d->ey[b], sizeof(Edge) * d->ney) == cudaSuccess;
    }
    if (ok) ok = cudaMalloc(&d->frames, sizeof(Frame2) * d->tiles.size()) == cudaSuccess;
    if (ok) ok = cudaMalloc(&d->tc, sizeof(TileC2) * d->tiles.size()) == cudaSuccess;
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
    cudaFree(d->B); cudaFree(d->Blo); cudaFree(d->C);
    for (int b = 0; b < 3; b++) { cudaFree(d->Ph[b]); cudaFree(d->Pl[b]); cudaFree(d->ex[b]); cudaFree(d->ey[b]); }
    cudaFree(d->frames);
    cudaFree(d->tc);
    cudaFree(d->d_doms);
    cudaFree(d->d_tiles);
    cudaFree(d->ckB);
    cudaFree(d->ckBlo);
    for (auto& g : d->graphs) cudaGraphExecDestroy(g.exec);
    delete d;
    *mixed_d2_slot(m) = nullptr;
}

// item's conserved state from primitive planes, U from P in FP64 (base_shll_2d.c:126-131)
int mixed2d_planes(MixedState* m, int item, MixedPlanes* out) {
    Mixed2D* d = get2(m);
    const Dom2& D = d->doms[item];
    out->hi = d->B;
    out->lo = d->Blo;
    out->base = D.base;
    out->plane = d->plane;
    out->n = (long)D.nx * D.ny;
    out->nv = 4;
    out->kahan = mixed_is_kahan(m);
    out->CV = D.CV;
    return SHLL_OK;
}

// the second-order step kernel of the batch's variant
template <bool VEC>
static void launch_o2v(bool kahan, bool pow2, int lim, int ntiles, cudaStream_t s, const Args2& A) {
    switch ((kahan ? 4 : 0) + (pow2 ? 2 : 0) + lim) {
        case 0: k_step2d_o2<false, false, 0, VEC><<<ntiles, NT2, kStepO2Smem, s>>>(A); break;
        case 1: k_step2d_o2<false, false, 1, VEC><<<ntiles, NT2, kStepO2Smem, s>>>(A); break;
        case 2: k_step2d_o2<false, true, 0, VEC><<<ntiles, NT2, kStepO2Smem, s>>>(A); break;
        case 3: k_step2d_o2<false, true, 1, VEC><<<ntiles, NT2, kStepO2Smem, s>>>(A); break;
        case 4: k_step2d_o2<true, false, 0, VEC><<<ntiles, NT2, kStepO2Smem, s>>>(A); break;
        case 5: k_step2d_o2<true, false, 1, VEC><<<ntiles, NT2, kStepO2Smem, s>>>(A); break;
        case 6: k_step2d_o2<true, true, 0, VEC><<<ntiles, NT2, kStepO2Smem, s>>>(A); break;
        default: k_step2d_o2<true, true, 1, VEC><<<ntiles, NT2, kStepO2Smem, s>>>(A); break;
    }
}
static void launch_o2(bool vec, bool kahan, bool pow2, int lim, int ntiles, cudaStream_t s, const Args2& A) {
    if (vec) launch_o2v<true>(kahan, pow2, lim, ntiles, s, A);
    else launch_o2v<false>(kahan, pow2, lim, ntiles, s, A);
}
// the two-step kernel of the batch's variant
template <bool VEC>
static void launch_step2(bool kahan, bool pow2, int ntiles, cudaStream_t s, const Args2& A) {
    if (kahan) {
        if (pow2) k_step2d2<true, true, VEC><<<ntiles, NT2, kStep2Smem, s>>>(A);
        else k_step2d2<true, false, VEC><<<ntiles, NT2, kStep2Smem, s>>>(A);
    } else {
        if (pow2) k_step2d2<false, true, VEC><<<ntiles, NT2, kStep2Smem, s>>>(A);
        else k_step2d2<false, false, VEC><<<ntiles, NT2, kStep2Smem, s>>>(A);
    }
}
// the first-order one-step kernel of the batch's variant
template <bool VEC>
static void launch_step1(bool kahan, bool pow2, int ntiles, cudaStream_t s, const Args2& A) {
    if (kahan) {
        if (pow2) k_step2d<true, true, VEC><<<ntiles, NTP, 0, s>>>(A);
        else k_step2d<true, false, VEC><<<ntiles, NTP, 0, s>>>(A);
    } else {
        if (pow2) k_step2d<false, true, VEC><<<ntiles, NTP, 0, s>>>(A);
        else k_step2d<false, false, VEC><<<ntiles, NTP, 0, s>>>(A);
    }
}

// the launches of one run on stream s: the opening fold, then per step k_step2d (k_step2d2 for two
// steps, k_step2d_o2 for second order) and a fold at the end of every window
static long issue_run2d(Mixed2D* d, MixedState* m, long maxsteps, cudaStream_t s) {
    Args2 A;
    memset(&A, 0, sizeof(A));
    A.doms = d->d_doms;
    A.tiles = d->d_tiles;
    A.frames = d->frames;
    A.tc = d->tc;
    A.B = d->B; A.Blo = d->Blo; A.C = d->C;
    for (int b = 0; b < 3; b++) {
        A.Ph[b] = d->Ph[b]; A.Pl[b] = d->Pl[b];
        A.ex[b] = d->ex[b]; A.ey[b] = d->ey[b];
    }
    A.plane = (int)d->plane;
    A.flag = mixed_flag_ptr(m);
    A.item_flags = mixed_item_flags_ptr(m);
    const bool kahan = mixed_is_kahan(m);
    const int ntiles = (int)d->tiles.size();
    long launches = 0;
    auto fold = [&](int s0, int win) {
        A.s0 = s0;
        A.win = win;
        if (kahan) k_fold2d<true><<<ntiles, NT, 0, s>>>(A);
        else k_fold2d<false><<<ntiles, NT, 0, s>>>(A);
        k_tileconst2d<<<ntiles, 64, 0, s>>>(A);
        launches += 2;
    };
    // lam_x and lam_y powers of two for every domain: the interface terms lam*Delta are exact
    bool pow2 = true;
    for (const Dom2& D : d->doms) {
        int ex;
        pow2 = pow2 && std::frexp(D.lamx, &ex) == 0.5 && std::frexp(D.lamy, &ex) == 0.5;
    }
    fold(0, 0);  // frames and C of the current state
    int s0 = 0;
    for (long st = 0; st < maxsteps;) {
        A.step = (int)st;
        A.s0 = s0;
        // two steps per launch inside a fold window, one for an odd remainder
        const long wend = std::min<long>(s0 + d->fold, maxsteps);
        const int k = d->kstep == 2 && wend - st >= 2 ? 2 : 1;
        if (d->order == 2) {
            launch_o2(d->vec, kahan, pow2, d->lim, ntiles, s, A);
        } else if (k == 2) {
            if (d->vec) launch_step2<true>(kahan, pow2, ntiles, s, A);
            else launch_step2<false>(kahan, pow2, ntiles, s, A);
        } else if (d->vec) {
            launch_step1<true>(kahan, pow2, ntiles, s, A);
        } else {
            launch_step1<false>(kahan, pow2, ntiles, s, A);
        }
        launches++;
        st += k;
        if (st == wend) {
            fold(s0, (int)(st - s0));
            s0 = (int)st;
        }
    }
    return launches;
}

// allows the two-step and second-order kernels their dynamic shared memory on the current device
// (before any capture)
static cudaError_t allow_step2_smem() {
    static unsigned long long done = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev >= 64 || (done & (1ull << dev))) return e;
    const void* ks[] = {(const void*)k_step2d2<false, false, false>, (const void*)k_step2d2<false, true, false>,
                        (const void*)k_step2d2<true, false, false>, (const void*)k_step2d2<true, true, false>,
                        (const void*)k_step2d2<false, false, true>, (const void*)k_step2d2<false, true, true>,
                        (const void*)k_step2d2<true, false, true>, (const void*)k_step2d2<true, true, true>};
    for (const void* k : ks) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kStep2Smem);
        if (e != cudaSuccess) return e;
    }
    const void* ko[] = {(const void*)k_step2d_o2<false, false, 0, false>, (const void*)k_step2d_o2<false, false, 1, false>,
                        (const void*)k_step2d_o2<false, true, 0, false>, (const void*)k_step2d_o2<false, true, 1, false>,
                        (const void*)k_step2d_o2<true, false, 0, false>, (const void*)k_step2d_o2<true, false, 1, false>,
                        (const void*)k_step2d_o2<true, true, 0, false>, (const void*)k_step2d_o2<true, true, 1, false>,
                        (const void*)k_step2d_o2<false, false, 0, true>, (const void*)k_step2d_o2<false, false, 1, true>,
                        (const void*)k_step2d_o2<false, true, 0, true>, (const void*)k_step2d_o2<false, true, 1, true>,
                        (const void*)k_step2d_o2<true, false, 0, true>, (const void*)k_step2d_o2<true, false, 1, true>,
                        (const void*)k_step2d_o2<true, true, 0, true>, (const void*)k_step2d_o2<true, true, 1, true>};
    for (const void* k : ko) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kStepO2Smem);
        if (e != cudaSuccess) return e;
    }
    done |= 1ull << dev;
    return cudaSuccess;
}

// Advances every domain by its own step count.  A run whose step counts and fold window occur a
// second time is captured into a CUDA graph, which later identical runs replay (the descriptors
// are uploaded before either); a run that occurs once is launched directly.
int mixed2d_run(MixedState* m, long nsteps, char* err, size_t len) {
    Mixed2D* d = get2(m);
    int count = 0;
    const shll_params* items = mixed_items(m, &count);
    long maxsteps = 0, updates = 0;
    std::vector<int> steps(count);
    for (int t = 0; t < count; t++) {
        const long s = nsteps >= 0 ? nsteps : shll_steps_for(&items[t]);
        d->doms[t].steps = (int)s;
        steps[t] = (int)s;
        maxsteps = std::max(maxsteps, s);
        updates += s * (long)d->doms[t].nx * d->doms[t].ny;
    }
    if (maxsteps == 0) return SHLL_OK;
    cudaStream_t s = mixed_stream(m);
    if (cudaMemcpyAsync(d->d_doms, d->doms.data(), sizeof(Dom2) * count, cudaMemcpyHostToDevice, s) != cudaSuccess) {
        snprintf(err, len, "2D descriptor upload failed");
        return SHLL_ERR_CUDA;
    }
    long launches = 0;
    cudaError_t e = allow_step2_smem();
    if (e != cudaSuccess) { snprintf(err, len, "kernel attribute: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    const bool replay = mixed_graph_replay_on(m) && s != nullptr;   // (the legacy stream cannot be captured)
    const int key = d->fold * 4 + d->kstep;
    Mixed2D::GraphEntry* hit = nullptr;
    if (replay)
        for (auto& g : d->graphs)
            if (g.steps == steps && g.fold == d->fold && g.kstep == d->kstep) hit = &g;
    if (hit) {
        e = cudaGraphLaunch(hit->exec, s);
        launches = hit->launches;
    } else {
        bool repeat = false, done = false;
        for (auto& k : d->seen) repeat = repeat || (k.first == steps && k.second == key);
        if (replay && !repeat) {
            if (d->seen.size() >= 8) d->seen.erase(d->seen.begin());
            d->seen.push_back({steps, key});
        }
        if (replay && repeat) {
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                const long l = issue_run2d(d, m, maxsteps, s);
                const cudaError_t ec = cudaStreamEndCapture(s, &graph);
                if (ec == cudaSuccess && graph && cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
                    if (d->graphs.size() >= 4) {
                        cudaGraphExecDestroy(d->graphs.front().exec);
                        d->graphs.erase(d->graphs.begin());
                    }
                    d->graphs.push_back({steps, d->fold, d->kstep, exec, l});
                    e = cudaGraphLaunch(exec, s);
                    launches = l;
                    done = true;
                }
                if (graph) cudaGraphDestroy(graph);
            }
            if (!done) cudaGetLastError();   // capture not possible here: launch directly
        }
        if (!done) {
            launches = issue_run2d(d, m, maxsteps, s);
            e = cudaGetLastError();
        }
    }
    shll_count_launches(launches);
    if (e != cudaSuccess) { snprintf(err, len, "2D step launch failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    mixed_add_updates(m, updates);
    return SHLL_OK;
}

int mixed2d_fold(MixedState* m) { return get2(m)->fold; }
int mixed2d_kstep(MixedState* m) { return get2(m)->kstep; }

// copies the stored state (FP64, or the FP32 value and compensation planes) to or from the checkpoint
int mixed2d_checkpoint(MixedState* m, bool restore, char* err, size_t len) {
    Mixed2D* d = get2(m);
    const bool kahan = mixed_is_kahan(m);
    const size_t nf = (size_t)4 * d->plane;
    const size_t vb = nf * (kahan ? sizeof(float) : sizeof(double));
    if (restore && !d->ckB) { snprintf(err, len, "no checkpoint taken"); return SHLL_ERR_STATE; }
    if (!restore && !d->ckB) {
        if (cudaMalloc(&d->ckB, vb) != cudaSuccess || (kahan && cudaMalloc(&d->ckBlo, nf * sizeof(float)) != cudaSuccess)) {
            cudaGetLastError();
            snprintf(err, len, "checkpoint allocation failed");
            return SHLL_ERR_NOMEM;
        }
    }
    cudaStream_t s = mixed_stream(m);
    cudaError_t e = restore ? cudaMemcpyAsync(d->B, d->ckB, vb, cudaMemcpyDeviceToDevice, s)
                            : cudaMemcpyAsync(d->ckB, d->B, vb, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && kahan)
        e = restore ? cudaMemcpyAsync(d->Blo, d->ckBlo, nf * sizeof(float), cudaMemcpyDeviceToDevice, s)
                    : cudaMemcpyAsync(d->ckBlo, d->Blo, nf * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) { snprintf(err, len, "checkpoint copy failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    return SHLL_OK;
}

// Autotuner of the 2D engine: times short runs of the batch (trial_steps steps, best of two, from a
// checkpoint restored after each) for the fold windows 16, 32, 64 and 128 steps (how many steps
// the increment pairs accumulate before the stored state absorbs them and the tiles get new frames)
// with one or two time steps per step launch, keeps the fastest for the batch and, process-wide,
// for its size class.
int mixed2d_autotune(MixedState* m, int trial_steps, char* err, size_t len) {
    Mixed2D* d = get2(m);
    if (trial_steps <= 0) trial_steps = 128;
    int rc = mixed2d_checkpoint(m, false, err, len);
    if (rc != SHLL_OK) return rc;
    cudaStream_t s = mixed_stream(m);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    mixed_set_tuning(m, true);
    const int keep = d->fold, keepk = d->kstep;
    int best = keep, bestk = keepk;
    float best_ms = 1e30f;
    for (int cand = 0; cand < 8; cand++) {
        const int f = 16 << (cand / 2), kk = 1 + cand % 2;
        if (f > trial_steps || (kk == 2 && d->order == 2)) continue;
        d->fold = f;
        d->kstep = kk;
        float ms = 1e30f;
        for (int rep = 0; rc == SHLL_OK && rep < 2; rep++) {
            rc = mixed2d_checkpoint(m, true, err, len);
            if (rc != SHLL_OK) break;
            cudaEventRecord(e0, s);
            rc = mixed2d_run(m, trial_steps, err, len);
            cudaEventRecord(e1, s);
            if (cudaEventSynchronize(e1) != cudaSuccess) { snprintf(err, len, "trial failed"); rc = SHLL_ERR_CUDA; }
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            ms = std::min(ms, t);
        }
        if (rc != SHLL_OK) break;
        if (ms < best_ms) { best_ms = ms; best = f; bestk = kk; }
    }
    mixed_set_tuning(m, false);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    d->fold = rc == SHLL_OK ? best : keep;
    d->kstep = rc == SHLL_OK ? bestk : keepk;
    const int rc2 = mixed2d_checkpoint(m, true, err, len);
    if (rc != SHLL_OK) return rc;
    if (rc2 != SHLL_OK) return rc2;
    std::lock_guard<std::mutex> lk(g_tune2d_mu);
    g_tune2d[tune2d_key(d->doms, mixed_is_kahan(m), d->order, d->lim)] = {best, bestk};
    return SHLL_OK;
}

int mixed2d_item_conserved(MixedState* m, int item, double* planes, char* err, size_t len) {
    Mixed2D* d = get2(m);
    const Dom2& D = d->doms[item];
    const size_t n = (size_t)D.nx * D.ny;
    cudaStream_t s = mixed_stream(m);
    for (int k = 0; k < 4; k++) {
        const size_t off = (size_t)k * d->plane + D.base;
        cudaError_t e;
        if (mixed_is_kahan(m)) {
            std::vector<float> h(n), l(n);
            e = cudaMemcpyAsync(h.data(), static_cast<float*>(d->B) + off, n * sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaMemcpyAsync(l.data(), d->Blo + off, n * sizeof(float), cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            for (size_t c = 0; c < n; c++) planes[k * n + c] = (double)h[c] + (double)l[c];
        } else {
            e = cudaMemcpyAsync(planes + k * n, static_cast<double*>(d->B) + off, n * sizeof(double),
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
    cudaStream_t s = mixed_stream(m);
    for (int k = 0; k < 4; k++) {
        const size_t off = (size_t)k * d->plane + D.base;
        cudaError_t e = mixed_is_kahan(m)
            ? device_pair_sums(static_cast<float*>(d->B) + off, d->Blo + off, 1, n, &out[k], s)
            : device_plane_sums(static_cast<double*>(d->B) + off, 64, 1, n, &out[k], s);
        if (e != cudaSuccess) { snprintf(err, len, "2D totals failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    }
    return SHLL_OK;
}

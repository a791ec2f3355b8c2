// Mixed-precision 1D SHLL engine: FP32 split fluxes in perturbation form, compensated FP32
// accumulation, FP64 (or FP32-pair) state folded once per sweep.
//
// Scheme (the arithmetic of base-c/base_shll.c:87-159 and of the x sweep of
// base-c/2nd_order_base_shll.c:203-459, re-associated as interface fluxes):
//   * Cells are grouped in chunks (one CTA each).  A chunk is computed over a window of its own
//     cells plus a halo of order*steps cells on each side (temporal blocking), so one launch
//     advances every chunk of every tube by a whole sweep of fold_steps steps, with no inter-CTA
//     waits.
//   * Every chunk has one frame: the FP64 state U* of an anchor cell at the start of the sweep
//     (the wall cell for the first and last chunk of a tube, else the centre cell) and the
//     split-flux coefficients derived from it.  Each window cell's split fluxes are evaluated in
//     FP32 as deviations from the frame (d fp = fp(U) - fp(U*), d fm likewise), with only
//     deviations as FP32 operands, so their rounding error scales with |U - U*| instead of |U|.
//   * The flux through interface j+1/2 is Fref + Delta_{j+1/2} (Fref = the anchor's physical
//     flux, which cancels inside a chunk); both neighbouring cells add the same FP32 value
//     lam*Delta with opposite signs (TwoSum into an FP32 value+compensation pair per cell).
//   * Neighbouring chunks evaluate their shared boundary interface in different frames, so the
//     two values differ by rounding.  Each chunk records the flux it applied at both of its
//     boundaries over the sweep; at the next load the right chunk's first cell receives
//     lam*sum(F_left chunk - F_right chunk), which makes the left chunk's value the one that
//     counts: mass, momentum and energy are conserved to the rounding of the FP64 state.
//   * At the end of a sweep the pair is added to the stored state: in FP64
//     (SHLL_PREC_MIXED_F64) or in FP32-pair arithmetic (SHLL_PREC_MIXED_KAHAN).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "mixed.h"
#include "mixed_common.cuh"
#include "shll_internal.h"

namespace {

constexpr int MW = 512;       // window capacity (cells) of one CTA
constexpr int MC = 1;         // cells per thread
constexpr int MT = MW / MC;   // threads per CTA

struct TubeP {
    long base;        // offset of cell 0 in the planes
    int n, order, limiter;
    int steps;        // steps of the current run
    int par;          // buffer holding the tube's state at the start of the run
    double gamma, R, CV, lam;
    float alpha;
    int lam_pow2;     // lam is a power of two: lam*Delta is exact in FP32
};

struct Chunk {
    int tube;
    int a, b;        // owned cells [a, b)
    int anc;         // anchor cell of the chunk's frame
    int id, idL, idR;  // this chunk's and its neighbours' ids (-1 if none), index of bsum
};

struct Frame1 {
    double U[3];      // anchor state
    double F[3];      // physical flux at the anchor = fp* + fm*
    double fpS1, fmS1;
    AnchorCoef c;
    float Uh[3], Ul[3];  // anchor as an FP32 pair
};

__device__ void make_frame(Frame1& f, const double U[3], const TubeP& tp) {
    double rho = U[0], m = U[1], E = U[2];
    double u = m / rho, e = E / rho;
    double T = (e - 0.5 * u * u) / tp.CV;
    double a = sqrt(tp.gamma * tp.R * T);
    double M = u / a, P = rho * tp.R * T;
    double Z1 = 0.5 * (M + 1.0), Z2 = 0.5 * a * (1.0 - M * M), Z3 = 0.5 * (M - 1.0);
    double F[3] = {m, m * u + P, u * (E + P)};
    for (int k = 0; k < 3; k++) {
        f.U[k] = U[k];
        f.F[k] = F[k];
        f.c.F[k] = (float)F[k];
        f.c.Uf[k] = (float)U[k];
        f.Uh[k] = (float)U[k];
        f.Ul[k] = (float)(U[k] - (double)f.Uh[k]);
    }
    f.fpS1 = F[1] * Z1 + m * Z2;
    f.fmS1 = -F[1] * Z3 - m * Z2;
    f.c.rho = (float)rho; f.c.u = (float)u; f.c.v = 0.f; f.c.e = (float)e; f.c.T = (float)T; f.c.a = (float)a;
    f.c.M = (float)M; f.c.P = (float)P; f.c.Z1 = (float)Z1; f.c.Z2 = (float)Z2;
    f.c.gR = (float)(tp.gamma * tp.R); f.c.R = (float)tp.R; f.c.cvinv = (float)(1.0 / tp.CV);
}

// reads the stored state of tube cell i as FP64 (F64 planes, or an FP32 pair)
template <bool KAHAN>
__device__ __forceinline__ double load_state(const void* __restrict__ hi, const float* __restrict__ lo, long idx) {
    if (KAHAN) return (double)static_cast<const float*>(hi)[idx] + (double)lo[idx];
    return static_cast<const double*>(hi)[idx];
}

// boundary flux sums of one chunk over a sweep: [side 0 = left interface, 1 = right][comp],
// each lam * sum over steps of the full flux (Fref + Delta) the chunk applied there
struct BSum {
    double s[2][3];
};

struct SweepArgs {
    const TubeP* tubes;
    const Chunk* chunks;
    void* hi[2];        // state planes of each buffer (double, or FP32 value)
    float* lo[2];       // FP32 compensation planes (Kahan)
    BSum* bsum[2];      // per chunk id, by sweep parity
    long plane;         // cells per plane (all tubes)
    int sweep, B;
    int* flag;
    int* item_flags;    // per tube (may be null)
};

// correction owed to the first owned cell of the chunk with id `right` by its left neighbour
// `left` for the sweep whose sums are in bs: lam*sum(F_left) - lam*sum(F_right) at their interface
__device__ __forceinline__ double boundary_correction(const BSum* bs, int left, int right, int k) {
    return bs[left].s[1][k] - bs[right].s[0][k];
}

struct Smem1 {
    Frame1 fr;
    alignas(16) float sfp[3][MW];
    alignas(16) float sfm[3][MW];
    float sTh[3][MT], sTl[3][MT];       // lam*Delta of each thread's last interface (FP32 pair)
    float wall[2][3][2];                // constant wall terms (order 1) for cell 0 / n-1
    double corr[2][3];                  // boundary corrections of cells a and b (previous sweep)
};

template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM>
__device__ void sweep_chunk(const SweepArgs& A, const Chunk& ch, const TubeP& tp, Smem1& S) {
    constexpr int R_ = ORDER;  // stencil reach per step
    Frame1& fr = S.fr;
    auto& sfp = S.sfp; auto& sfm = S.sfm; auto& sTh = S.sTh; auto& sTl = S.sTl; auto& wall = S.wall;

    const int tid = threadIdx.x;
    const int n = tp.n;
    const int steps = min(A.B, tp.steps - A.sweep * A.B);
    if (steps <= 0) return;
    const int H = R_ * steps;
    const int ws = max(0, ch.a - H), we = min(n, ch.b + H), L = we - ws;
    const int pa = ch.a - ws, pb = ch.b - ws;  // first owned / one past the last owned, window coords
    const int inb = (tp.par + A.sweep) & 1, outb = inb ^ 1;
    // (selects rather than indexing the parameter arrays, which would copy them to local memory)
    const void* hin = inb ? A.hi[1] : A.hi[0];
    const float* lin = inb ? A.lo[1] : A.lo[0];
    const long base = tp.base;
    const long P = A.plane;
    const double lam = tp.lam;
    const float lamh = (float)lam, laml = (float)(lam - (double)lamh);

    if (L > MW) {  // host guarantees this never happens; refuse rather than overrun
        if (tid == 0) atomicOr(A.flag, SHLL_FLAG_BADARG);
        return;
    }
    // corrections of the previous sweep for cell a (from the left neighbour) and cell b (the right
    // neighbour's first cell, which lies in this window's halo)
    if (tid < 6) {
        const int side = tid / 3, k = tid % 3;
        double c = 0.0;
        if (A.sweep > 0) {
            const BSum* bs = ((A.sweep - 1) & 1) ? A.bsum[1] : A.bsum[0];
            if (side == 0 && ch.idL >= 0) c = boundary_correction(bs, ch.idL, ch.id, k);
            if (side == 1 && ch.idR >= 0) c = boundary_correction(bs, ch.id, ch.idR, k);
        }
        S.corr[side][k] = c;
    }
    __syncthreads();
    if (tid == 0) {
        double U[3];
        for (int k = 0; k < 3; k++) {
            U[k] = load_state<KAHAN>(hin, lin, k * P + base + ch.anc);
            if (ch.anc == ch.a) U[k] += S.corr[0][k];
            if (ch.anc == ch.b) U[k] += S.corr[1][k];
        }
        make_frame(fr, U, tp);
    }
    __syncthreads();
    if (tid < 6 && ORDER == 1) {
        // reflective walls: constant parts of the wall-cell increments
        // cell 0:   lam*F_{-1/2} - lam*Fref = (-lam F0, lam (2 fmS1 - F1), -lam F2) (+2 lam dfm1_0)
        // cell n-1: lam*Fref - lam*F_{n-1/2} = (lam F0, lam (F1 - 2 fpS1), lam F2) (-2 lam dfp1_{n-1})
        const int bnd = tid / 3, k = tid % 3;
        double w = bnd == 0 ? (k == 1 ? lam * (2.0 * fr.fmS1 - fr.F[1]) : -lam * fr.F[k])
                            : (k == 1 ? lam * (fr.F[1] - 2.0 * fr.fpS1) : lam * fr.F[k]);
        split2(w, wall[bnd][k][0], wall[bnd][k][1]);
    }

    // ---- load the window as deviations from the frame ----
    const int w0 = tid * MC;
    float dh[MC][3], dl[MC][3];
#pragma unroll
    for (int q = 0; q < MC; q++) {
        const int w = w0 + q;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            dh[q][k] = 0.f; dl[q][k] = 0.f;
            if (w < L) {
                const long idx = k * P + base + ws + w;
                const bool corrected = w == pa || w == pb;  // cells owed a boundary correction
                if (KAHAN) {
                    const float h = static_cast<const float*>(hin)[idx], l = lin[idx];
                    if (corrected) {
                        const double d = ((double)h - fr.U[k]) + (double)l + S.corr[w == pa ? 0 : 1][k];
                        split2(d, dh[q][k], dl[q][k]);
                    } else {
                        ff_sub(h, l, fr.Uh[k], fr.Ul[k], dh[q][k], dl[q][k]);
                    }
                } else {
                    double d = static_cast<const double*>(hin)[idx] - fr.U[k];
                    if (corrected) d += S.corr[w == pa ? 0 : 1][k];
                    split2(d, dh[q][k], dl[q][k]);
                }
            }
        }
    }
    // flux sums at the chunk's two boundary interfaces (kept by the threads that apply them)
    float bh[2][3] = {{0, 0, 0}, {0, 0, 0}}, bl[2][3] = {{0, 0, 0}, {0, 0, 0}};
    const bool hasL = ch.idL >= 0, hasR = ch.idR >= 0;
    // loop-invariant roles of this thread's cells
    bool in_ok[MC], out_ok[MC], sp0[MC], sm0[MC], special[MC];
#pragma unroll
    for (int q = 0; q < MC; q++) {
        const int w = w0 + q, i = ws + w;
        in_ok[q] = i > 0 && w > 0 && w < L;
        out_ok[q] = i < n - 1 && w < L - 1;
        sp0[q] = i == 0 || i == n - 1;          // dfp of cell i is zero (edge cell)
        sm0[q] = i + 1 == n - 1;                // dfm of cell i+1 is zero
        special[q] = w < L && (i == 0 || i == n - 1 || (w == pa && hasL) || (w == pb - 1 && hasR));
    }

    for (int s = 0; s < steps; s++) {
        // ---- A: split-flux deviations ----
        float fp[MC][3], fm[MC][3];
#pragma unroll
        for (int q = 0; q < MC; q++) {
            float d[3];
#pragma unroll
            for (int k = 0; k < 3; k++) d[k] = __fadd_rn(dh[q][k], dl[q][k]);
            dflux1(fr.c, d, fp[q], fm[q]);
        }
#pragma unroll
        for (int q = 0; q < MC; q++)
#pragma unroll
            for (int k = 0; k < 3; k++) { sfp[k][w0 + q] = fp[q][k]; sfm[k][w0 + q] = fm[q][k]; }
        __syncthreads();
        // ---- B: interface terms lam*Delta_{j+1/2}, j = w0..w0+MC-1 ----
        float th[MC][3], tl[MC][3];
        float pl[3], pr[2][3], mr[2][3];
        {   // neighbours' values (clamped at the window ends, whose cells are in the halo)
            const int cl = max(w0 - 1, 0), cr0 = min(w0 + MC, MW - 1), cr1 = min(w0 + MC + 1, MW - 1);
#pragma unroll
            for (int k = 0; k < 3; k++) {
                if (ORDER == 2) { pl[k] = sfp[k][cl]; pr[0][k] = sfp[k][cr0]; mr[1][k] = sfm[k][cr1]; }
                mr[0][k] = sfm[k][cr0];
            }
        }
#pragma unroll
        for (int q = 0; q < MC; q++) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                float Dl;
                const float p1 = fp[q][k];
                const float m2 = q + 1 < MC ? fm[q + 1][k] : mr[0][k];
                if (ORDER == 1) {
                    Dl = __fadd_rn(p1, m2);
                } else {
                    const float p0 = q > 0 ? fp[q - 1][k] : pl[k];
                    const float p2 = q + 1 < MC ? fp[q + 1][k] : pr[0][k];
                    const float m1 = fm[q][k];
                    const float m3 = q + 2 < MC ? fm[q + 2][k] : mr[q + 2 - MC][k];
                    const float sp = sp0[q] ? 0.f : slope_f<LIM>(p0, p1, p2, tp.alpha);
                    const float sm = sm0[q] ? 0.f : slope_f<LIM>(m1, m2, m3, tp.alpha);
                    Dl = __fadd_rn(__fadd_rn(__fadd_rn(p1, __fmul_rn(0.5f, sp)), m2), -__fmul_rn(0.5f, sm));
                }
                th[q][k] = __fmul_rn(lamh, Dl);
                tl[q][k] = LAM_POW2 ? 0.f : __fadd_rn(__fmaf_rn(lamh, Dl, -th[q][k]), __fmul_rn(laml, Dl));
            }
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            sTh[k][tid] = th[MC - 1][k];
            if (!LAM_POW2) sTl[k][tid] = tl[MC - 1][k];
        }
        __syncthreads();
        // ---- C: accumulate lam*(F_{i-1/2} - F_{i+1/2}) per cell ----
        const int tl_ = max(tid - 1, 0);
#pragma unroll
        for (int q = 0; q < MC; q++) {
#pragma unroll
            for (int k = 0; k < 3; k++) {
                float ih = q > 0 ? th[q - 1][k] : sTh[k][tl_];
                float il = LAM_POW2 ? 0.f : (q > 0 ? tl[q - 1][k] : sTl[k][tl_]);
                ih = in_ok[q] ? ih : 0.f;
                il = in_ok[q] ? il : 0.f;
                const float oh = out_ok[q] ? th[q][k] : 0.f;
                const float ol = out_ok[q] ? tl[q][k] : 0.f;
                two_sum_acc(dh[q][k], dl[q][k], ih);
                two_sum_acc(dh[q][k], dl[q][k], -oh);
                if (!LAM_POW2) dl[q][k] = __fadd_rn(dl[q][k], __fadd_rn(il, -ol));
                if (special[q]) {
                    const int w = w0 + q, i = ws + w;
                    float& h = dh[q][k];
                    float& l = dl[q][k];
                    if (w == pa && hasL) { two_sum_acc(bh[0][k], bl[0][k], ih); bl[0][k] = __fadd_rn(bl[0][k], il); }
                    if (w == pb - 1 && hasR) { two_sum_acc(bh[1][k], bl[1][k], oh); bl[1][k] = __fadd_rn(bl[1][k], ol); }
                    if (i == 0 || i == n - 1) {
                        if (ORDER == 1) {
                            const int bnd = i == 0 ? 0 : 1;
                            two_sum_acc(h, l, wall[bnd][k][0]); l = __fadd_rn(l, wall[bnd][k][1]);
                            if (k == 1) {  // +2 lam dfm1_0 at the left wall, -2 lam dfp1_{n-1} at the right
                                const float v = i == 0 ? __fmul_rn(2.f, fm[q][1]) : -__fmul_rn(2.f, fp[q][1]);
                                const float vh = __fmul_rn(lamh, v);
                                const float vl = __fadd_rn(__fmaf_rn(lamh, v, -vh), __fmul_rn(laml, v));
                                two_sum_acc(h, l, vh); l = __fadd_rn(l, vl);
                            }
                        } else {  // outflow: F_{-1/2} = Fref + dfp_0 + dfm_0 (and likewise at n-1)
                            float v = __fadd_rn(fp[q][k], fm[q][k]);
                            if (i == n - 1) v = -v;
                            const float vh = __fmul_rn(lamh, v);
                            const float vl = __fadd_rn(__fmaf_rn(lamh, v, -vh), __fmul_rn(laml, v));
                            two_sum_acc(h, l, vh); l = __fadd_rn(l, vl);
                        }
                    }
                }
            }
        }
    }
    // ---- boundary flux sums of this sweep (full flux: steps * lam * Fref + sum lam*Delta) ----
    BSum* bout = ((A.sweep & 1) ? A.bsum[1] : A.bsum[0]) + ch.id;
#pragma unroll
    for (int q = 0; q < MC; q++) {
        const int w = w0 + q;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (w == pa && hasL) bout->s[0][k] = steps * lam * fr.F[k] + ((double)bh[0][k] + (double)bl[0][k]);
            if (w == pb - 1 && hasR) bout->s[1][k] = steps * lam * fr.F[k] + ((double)bh[1][k] + (double)bl[1][k]);
        }
    }

    // ---- fold the owned cells into the stored state ----
    int bad = 0;
    void* hout = outb ? A.hi[1] : A.hi[0];
    float* lout = outb ? A.lo[1] : A.lo[0];
#pragma unroll
    for (int q = 0; q < MC; q++) {
        const int w = w0 + q;
        if (w < pa || w >= pb) continue;
        double uu[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const long idx = k * P + base + ws + w;
            if (KAHAN) {
                float oh, ol;
                ff_add(fr.Uh[k], fr.Ul[k], dh[q][k], dl[q][k], oh, ol);
                static_cast<float*>(hout)[idx] = oh;
                lout[idx] = ol;
                uu[k] = (double)oh;
            } else {
                const double v = fr.U[k] + ((double)dh[q][k] + (double)dl[q][k]);
                static_cast<double*>(hout)[idx] = v;
                uu[k] = v;
            }
        }
        const float r = (float)uu[0], m = (float)uu[1], E = (float)uu[2];
        const float eint = __fadd_rn(E, -__fmul_rn(0.5f, __fdividef(__fmul_rn(m, m), r)));
        bad |= !(r > 0.f) || !(eint > 0.f);
    }
    if (bad) {
        atomicOr(A.flag, SHLL_FLAG_NONPOSITIVE);
        if (A.item_flags) atomicOr(&A.item_flags[ch.tube], SHLL_FLAG_NONPOSITIVE);
    }
}

template <bool KAHAN>
__global__ void __launch_bounds__(MT) k_sweep1d(SweepArgs A) {
    __shared__ Smem1 S;
    const Chunk ch = A.chunks[blockIdx.x];
    const TubeP tp = A.tubes[ch.tube];
    const bool pow2 = tp.lam_pow2;
    if (tp.order == 2) {
        if (tp.limiter == 1) {
            if (pow2) sweep_chunk<2, KAHAN, true, 1>(A, ch, tp, S);
            else sweep_chunk<2, KAHAN, false, 1>(A, ch, tp, S);
        } else {
            if (pow2) sweep_chunk<2, KAHAN, true, 0>(A, ch, tp, S);
            else sweep_chunk<2, KAHAN, false, 0>(A, ch, tp, S);
        }
    } else {
        if (pow2) sweep_chunk<1, KAHAN, true, 0>(A, ch, tp, S);
        else sweep_chunk<1, KAHAN, false, 0>(A, ch, tp, S);
    }
}

// Applies the last sweep's boundary corrections of a run to the first owned cell of every chunk
// that has a left neighbour (the state buffer that holds the tube after the run).
template <bool KAHAN>
__global__ void k_fixup1d(SweepArgs A, int nchunks) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nchunks) return;
    const Chunk ch = A.chunks[c];
    const TubeP tp = A.tubes[ch.tube];
    if (ch.idL < 0 || tp.steps <= 0) return;
    const int sweeps = (tp.steps + A.B - 1) / A.B;
    const BSum* bs = ((sweeps - 1) & 1) ? A.bsum[1] : A.bsum[0];
    const int buf = (tp.par + sweeps) & 1;
    for (int k = 0; k < 3; k++) {
        const long idx = k * A.plane + tp.base + ch.a;
        const double corr = boundary_correction(bs, ch.idL, ch.id, k);
        if (KAHAN) {
            float* h = static_cast<float*>(buf ? A.hi[1] : A.hi[0]);
            float* l = buf ? A.lo[1] : A.lo[0];
            const double v = ((double)h[idx] + (double)l[idx]) + corr;
            split2(v, h[idx], l[idx]);
        } else {
            static_cast<double*>(buf ? A.hi[1] : A.hi[0])[idx] += corr;
        }
    }
}

}  // namespace

// ------------------------------------------------------------------------------------------
// host side
struct MixedState {
    int dim = 1, nitems = 0, precision = SHLL_PREC_MIXED_F64, B = 16;
    bool kahan = false;
    cudaStream_t stream = nullptr;
    std::vector<shll_params> items;
    std::vector<TubeP> tubes;          // host copy
    std::vector<int> par;              // per tube: buffer holding its current state
    long plane = 0;                    // cells per plane
    void* hi[2] = {nullptr, nullptr};
    float* lo[2] = {nullptr, nullptr};
    TubeP* d_tubes = nullptr;
    Chunk* d_chunks = nullptr;
    std::vector<Chunk> chunks;         // sorted by the steps of their tube (descending)
    int* d_flag = nullptr;
    int* d_item_flags = nullptr;       // per item
    BSum* bsum[2] = {nullptr, nullptr};  // boundary flux sums per chunk id, by sweep parity
    long cell_updates = 0;
    // device checkpoint (shll_checkpoint)
    void* ck_hi[2] = {nullptr, nullptr};
    float* ck_lo[2] = {nullptr, nullptr};
    std::vector<int> ck_par;
    long ck_updates = 0;
    // 2D engine (mixed2d.cu)
    void* d2 = nullptr;
};

// owned cells per chunk: the window (MW) minus the halo on both sides; SHLL_MIXED_CHUNK (cells)
// may lower it to put more CTAs on each SM
static int chunk_owned(int order, int B) {
    int S = MW - 2 * order * B;
    if (const char* e = getenv("SHLL_MIXED_CHUNK")) {
        int v = atoi(e);
        if (v >= 4 * order * B && v < S) S = v;
    }
    return S;
}

// Chunks of every tube.  A tube has at least two chunks; the first chunk's frame is anchored
// at the left wall cell and the last chunk's at the right wall cell, so that a wall region
// still equal to its wall cell has exactly zero split-flux deviations (as in the reference, a
// gas at rest next to a wall stays exactly at rest); interior chunks anchor at their centre.
static void build_chunks(MixedState* m) {
    m->chunks.clear();
    for (int t = 0; t < m->nitems; t++) {
        const TubeP& tp = m->tubes[t];
        const int n = tp.n;
        const int S = chunk_owned(tp.order, m->B);
        int k = n <= MW ? 2 : (n + S - 1) / S;
        if (k > n) k = n;
        std::vector<int> edges(k + 1), anc(k);
        for (int c = 0; c <= k; c++) edges[c] = (int)((long)n * c / k);
        for (int c = 0; c < k; c++) anc[c] = c == 0 ? 0 : (c == k - 1 ? n - 1 : (edges[c] + edges[c + 1]) / 2);
        const int id0 = (int)m->chunks.size();
        for (int c = 0; c < k; c++)
            m->chunks.push_back({t, edges[c], edges[c + 1], anc[c], id0 + c, c > 0 ? id0 + c - 1 : -1,
                                 c + 1 < k ? id0 + c + 1 : -1});
    }
}

static int alloc_mixed(MixedState* m, char* err, size_t len) {
    const size_t cells = (size_t)m->plane * 3;
    for (int b = 0; b < 2; b++) {
        if (cudaMalloc(&m->hi[b], cells * (m->kahan ? sizeof(float) : sizeof(double))) != cudaSuccess) {
            snprintf(err, len, "cudaMalloc of %zu state values failed", cells);
            return SHLL_ERR_NOMEM;
        }
        if (m->kahan && cudaMalloc(&m->lo[b], cells * sizeof(float)) != cudaSuccess) {
            snprintf(err, len, "cudaMalloc of compensation planes failed");
            return SHLL_ERR_NOMEM;
        }
    }
    for (int b = 0; b < 2; b++) {
        if (cudaMalloc(&m->bsum[b], sizeof(BSum) * m->chunks.size()) != cudaSuccess ||
            cudaMemset(m->bsum[b], 0, sizeof(BSum) * m->chunks.size()) != cudaSuccess) {
            snprintf(err, len, "cudaMalloc of boundary sums failed");
            return SHLL_ERR_NOMEM;
        }
    }
    if (cudaMalloc(&m->d_item_flags, sizeof(int) * m->nitems) != cudaSuccess ||
        cudaMemset(m->d_item_flags, 0, sizeof(int) * m->nitems) != cudaSuccess) {
        snprintf(err, len, "cudaMalloc of item flags failed");
        return SHLL_ERR_NOMEM;
    }
    if (cudaMalloc(&m->d_tubes, sizeof(TubeP) * m->nitems) != cudaSuccess ||
        cudaMalloc(&m->d_flag, sizeof(int)) != cudaSuccess || cudaMemset(m->d_flag, 0, sizeof(int)) != cudaSuccess) {
        snprintf(err, len, "cudaMalloc of descriptors failed");
        return SHLL_ERR_NOMEM;
    }
    return SHLL_OK;
}

// FP64 reference constants of one item (the reference's REAL = double values)
static void item_consts(const shll_params& p, double* CV, double* lam, double* lamy) {
    double R = p.R, g = p.gamma;
    *CV = R / (g - 1.0);
    double dx = p.lx / p.nx, dy = p.ly / (p.dim == 2 ? p.ny : 1);
    double dt = (p.cfl / (R + 1)) * dx;
    *lam = p.cfl / (R + 1);
    *lamy = dt / dy;
}

MixedState* mixed2d_attach(MixedState* m, char* err, size_t len);  // mixed2d.cu
void mixed2d_detach(MixedState* m);
int mixed2d_load(MixedState* m, int item, const double* prim, char* err, size_t len);
int mixed2d_run(MixedState* m, long nsteps, char* err, size_t len);
int mixed2d_item_conserved(MixedState* m, int item, double* planes, char* err, size_t len);
int mixed2d_totals(MixedState* m, int item, double* out, char* err, size_t len);

MixedState* mixed_create_batch(const shll_params* items, int count, cudaStream_t s, char* err, size_t len) {
    if (count <= 0 || !items) { snprintf(err, len, "empty batch"); return nullptr; }
    MixedState* m = new MixedState();
    m->stream = s;
    m->nitems = count;
    m->items.assign(items, items + count);
    m->dim = items[0].dim;
    m->precision = items[0].precision;
    m->kahan = m->precision == SHLL_PREC_MIXED_KAHAN;
    int fold = items[0].fold_steps > 0 ? items[0].fold_steps : 16;
    for (int t = 0; t < count; t++) {
        if (items[t].dim != m->dim || items[t].precision != m->precision) {
            snprintf(err, len, "batch items must share dim and precision");
            delete m;
            return nullptr;
        }
        if (items[t].precision != SHLL_PREC_MIXED_F64 && items[t].precision != SHLL_PREC_MIXED_KAHAN) {
            snprintf(err, len, "the mixed engine takes MIXED_F64 or MIXED_KAHAN items");
            delete m;
            return nullptr;
        }
    }
    if (m->dim == 2) {
        m->B = fold;
        if (cudaMalloc(&m->d_flag, sizeof(int)) != cudaSuccess || cudaMemset(m->d_flag, 0, sizeof(int)) != cudaSuccess ||
            cudaMalloc(&m->d_item_flags, sizeof(int) * count) != cudaSuccess ||
            cudaMemset(m->d_item_flags, 0, sizeof(int) * count) != cudaSuccess) {
            snprintf(err, len, "cudaMalloc of the error flags failed");
            mixed_destroy(m);
            return nullptr;
        }
        if (!mixed2d_attach(m, err, len)) { mixed_destroy(m); return nullptr; }
        return m;
    }
    // sweep length: the fold interval, capped so that a chunk keeps at least half its window
    m->B = std::min(fold, MW / 16);
    long off = 0;
    for (int t = 0; t < count; t++) {
        const shll_params& p = items[t];
        TubeP tp;
        memset(&tp, 0, sizeof(tp));
        tp.base = off;
        tp.n = p.nx;
        tp.order = p.order;
        tp.limiter = p.limiter;
        tp.gamma = p.gamma;
        tp.R = p.R;
        double lamy;
        item_consts(p, &tp.CV, &tp.lam, &lamy);
        tp.alpha = (float)p.mc_alpha;
        {
            int ex;
            tp.lam_pow2 = std::frexp(tp.lam, &ex) == 0.5 && ex > -100 && ex < 100;
        }
        tp.steps = 0;
        tp.par = 0;
        m->tubes.push_back(tp);
        off += p.nx;
    }
    m->plane = off;
    m->par.assign(count, 0);
    build_chunks(m);
    int rc = alloc_mixed(m, err, len);
    if (rc == SHLL_OK && cudaMalloc(&m->d_chunks, sizeof(Chunk) * m->chunks.size()) != cudaSuccess) rc = SHLL_ERR_NOMEM;
    if (rc != SHLL_OK) {
        mixed_destroy(m);
        return nullptr;
    }
    return m;
}

MixedState* mixed_create(const shll_params* p, double, double, double, cudaStream_t s, char* err, size_t len) {
    return mixed_create_batch(p, 1, s, err, len);
}

void mixed_destroy(MixedState* m) {
    if (!m) return;
    if (m->d2) mixed2d_detach(m);
    for (int b = 0; b < 2; b++) {
        cudaFree(m->hi[b]); cudaFree(m->lo[b]); cudaFree(m->ck_hi[b]); cudaFree(m->ck_lo[b]);
    }
    cudaFree(m->d_tubes);
    cudaFree(m->d_chunks);
    cudaFree(m->bsum[0]);
    cudaFree(m->bsum[1]);
    cudaFree(m->d_flag);
    cudaFree(m->d_item_flags);
    delete m;
}

void mixed_set_stream(MixedState* m, cudaStream_t s) { m->stream = s; }

int mixed_flags(MixedState* m) {
    int h = 0;
    int* f = m->d_flag;
    if (!f) return 0;
    cudaMemcpyAsync(&h, f, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
    cudaStreamSynchronize(m->stream);
    return h;
}

// writes item t's conserved state (FP64, from primitive planes computed as the FP64 reference
// does: Compute_U_from_P of base_shll.c:76-80) into buffer par[t]
static int load_tube(MixedState* m, int t, const double* prim, char* err, size_t len) {
    const TubeP& tp = m->tubes[t];
    const int n = tp.n;
    const double CV = tp.CV;
    std::vector<double> U(3 * (size_t)n);
    for (int i = 0; i < n; i++) {
        double p0 = prim[i], p1 = prim[n + i], p2 = prim[2 * n + i];
        U[i] = p0;
        U[n + i] = p0 * p1;
        U[2 * n + i] = p0 * (p2 * CV + 0.5 * p1 * p1);
    }
    m->par[t] = 0;
    for (int k = 0; k < 3; k++) {
        const size_t off = (size_t)k * m->plane + tp.base;
        if (m->kahan) {
            std::vector<float> h(n), l(n);
            for (int i = 0; i < n; i++) {
                h[i] = (float)U[k * n + i];
                l[i] = (float)(U[k * n + i] - (double)h[i]);
            }
            if (cudaMemcpyAsync(static_cast<float*>(m->hi[0]) + off, h.data(), n * sizeof(float), cudaMemcpyHostToDevice, m->stream) != cudaSuccess ||
                cudaMemcpyAsync(m->lo[0] + off, l.data(), n * sizeof(float), cudaMemcpyHostToDevice, m->stream) != cudaSuccess ||
                cudaStreamSynchronize(m->stream) != cudaSuccess) {
                snprintf(err, len, "state upload failed");
                return SHLL_ERR_CUDA;
            }
        } else {
            if (cudaMemcpyAsync(static_cast<double*>(m->hi[0]) + off, U.data() + (size_t)k * n, n * sizeof(double),
                                cudaMemcpyHostToDevice, m->stream) != cudaSuccess) {
                snprintf(err, len, "state upload failed");
                return SHLL_ERR_CUDA;
            }
        }
    }
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) { snprintf(err, len, "state upload failed"); return SHLL_ERR_CUDA; }
    return SHLL_OK;
}

int mixed_load(MixedState* m, const double* prim, char* err, size_t len) {
    cudaMemsetAsync(m->d_flag, 0, sizeof(int), m->stream);
    cudaMemsetAsync(m->d_item_flags, 0, sizeof(int) * m->nitems, m->stream);
    if (m->dim == 2) return mixed2d_load(m, 0, prim, err, len);
    return load_tube(m, 0, prim, err, len);
}

int mixed_load_all(MixedState* m, char* err, size_t len) {
    cudaMemsetAsync(m->d_flag, 0, sizeof(int), m->stream);
    cudaMemsetAsync(m->d_item_flags, 0, sizeof(int) * m->nitems, m->stream);
    for (int t = 0; t < m->nitems; t++) {
        const shll_params& p = m->items[t];
        std::vector<double> prim((size_t)(p.dim == 2 ? 4 : 3) * p.nx * (p.dim == 2 ? p.ny : 1));
        shll_ic_fill(&p, 64, prim.data());
        int rc = m->dim == 2 ? mixed2d_load(m, t, prim.data(), err, len) : load_tube(m, t, prim.data(), err, len);
        if (rc != SHLL_OK) return rc;
    }
    return SHLL_OK;
}

// advances every tube by `steps[t]` steps (one launch per sweep of B steps)
static int run_tubes(MixedState* m, const std::vector<long>& steps, char* err, size_t len) {
    long maxsteps = 0;
    for (int t = 0; t < m->nitems; t++) {
        m->tubes[t].steps = (int)steps[t];
        m->tubes[t].par = m->par[t];
        maxsteps = std::max(maxsteps, steps[t]);
    }
    if (maxsteps == 0) return SHLL_OK;
    // chunks ordered by their tube's sweep count, so launch k covers a prefix of the list
    std::vector<Chunk> order = m->chunks;
    std::stable_sort(order.begin(), order.end(), [&](const Chunk& x, const Chunk& y) {
        return m->tubes[x.tube].steps > m->tubes[y.tube].steps;
    });
    if (cudaMemcpyAsync(m->d_tubes, m->tubes.data(), sizeof(TubeP) * m->nitems, cudaMemcpyHostToDevice, m->stream) != cudaSuccess ||
        cudaMemcpyAsync(m->d_chunks, order.data(), sizeof(Chunk) * order.size(), cudaMemcpyHostToDevice, m->stream) != cudaSuccess) {
        snprintf(err, len, "descriptor upload failed");
        return SHLL_ERR_CUDA;
    }
    const long nsweeps = (maxsteps + m->B - 1) / m->B;
    // active[k] = chunks whose tube still has sweep k (suffix sum of a histogram of sweep counts)
    std::vector<int> active(nsweeps + 1, 0);
    for (const Chunk& c : order) active[(m->tubes[c.tube].steps + m->B - 1) / m->B]++;
    for (long k = nsweeps - 1; k >= 0; k--) active[k] += active[k + 1];
    std::vector<int> launch(nsweeps);
    for (long k = 0; k < nsweeps; k++) launch[k] = active[k + 1];
    SweepArgs A;
    A.tubes = m->d_tubes;
    A.chunks = m->d_chunks;
    A.hi[0] = m->hi[0]; A.hi[1] = m->hi[1];
    A.lo[0] = m->lo[0]; A.lo[1] = m->lo[1];
    A.bsum[0] = m->bsum[0]; A.bsum[1] = m->bsum[1];
    A.plane = m->plane;
    A.B = m->B;
    A.flag = m->d_flag;
    A.item_flags = m->d_item_flags;
    A.sweep = 0;
    shll_count_launches(nsweeps + 1);
    for (long k = 0; k < nsweeps; k++) {
        A.sweep = (int)k;
        if (launch[k] == 0) continue;
        if (m->kahan) k_sweep1d<true><<<launch[k], MT, 0, m->stream>>>(A);
        else k_sweep1d<false><<<launch[k], MT, 0, m->stream>>>(A);
    }
    const int nch = (int)order.size();
    if (m->kahan) k_fixup1d<true><<<(nch + 127) / 128, 128, 0, m->stream>>>(A, nch);
    else k_fixup1d<false><<<(nch + 127) / 128, 128, 0, m->stream>>>(A, nch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { snprintf(err, len, "sweep launch failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    for (int t = 0; t < m->nitems; t++) {
        long sw = (steps[t] + m->B - 1) / m->B;
        m->par[t] = (int)((m->par[t] + sw) & 1);
        m->cell_updates += steps[t] * (long)m->tubes[t].n;
    }
    return SHLL_OK;
}

int mixed_step(MixedState* m, long nsteps, char* err, size_t len) {
    if (m->dim == 2) return mixed2d_run(m, nsteps, err, len);
    std::vector<long> steps(m->nitems);
    for (int t = 0; t < m->nitems; t++) steps[t] = nsteps >= 0 ? nsteps : shll_steps_for(&m->items[t]);
    return run_tubes(m, steps, err, len);
}

long mixed_cell_updates(const MixedState* m) { return m->cell_updates; }

// FP64 conserved planes of one item (rho, rho*u, E)
static int tube_conserved(MixedState* m, int t, double* planes, char* err, size_t len) {
    const TubeP& tp = m->tubes[t];
    const int n = tp.n, b = m->par[t];
    for (int k = 0; k < 3; k++) {
        const size_t off = (size_t)k * m->plane + tp.base;
        cudaError_t e;
        if (m->kahan) {
            std::vector<float> h(n), l(n);
            e = cudaMemcpyAsync(h.data(), static_cast<float*>(m->hi[b]) + off, n * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
            if (e == cudaSuccess) e = cudaMemcpyAsync(l.data(), m->lo[b] + off, n * sizeof(float), cudaMemcpyDeviceToHost, m->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
            for (int i = 0; i < n; i++) planes[(size_t)k * n + i] = (double)h[i] + (double)l[i];
        } else {
            e = cudaMemcpyAsync(planes + (size_t)k * n, static_cast<double*>(m->hi[b]) + off, n * sizeof(double),
                                cudaMemcpyDeviceToHost, m->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        }
        if (e != cudaSuccess) { snprintf(err, len, "state download failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    }
    return SHLL_OK;
}

int mixed_item_conserved(MixedState* m, int item, double* planes, char* err, size_t len) {
    if (item < 0 || item >= m->nitems) { snprintf(err, len, "item %d out of range", item); return SHLL_ERR_ARG; }
    if (m->dim == 2) return mixed2d_item_conserved(m, item, planes, err, len);
    return tube_conserved(m, item, planes, err, len);
}

int mixed_item_primitives(MixedState* m, int item, double* rho, double* u, double* v, double* T, char* err, size_t len) {
    if (item < 0 || item >= m->nitems) { snprintf(err, len, "item %d out of range", item); return SHLL_ERR_ARG; }
    const shll_params& p = m->items[item];
    const size_t n = (size_t)p.nx * (p.dim == 2 ? p.ny : 1);
    const int nv = p.dim == 2 ? 4 : 3;
    std::vector<double> U(nv * n);
    int rc = mixed_item_conserved(m, item, U.data(), err, len);
    if (rc != SHLL_OK) return rc;
    const double CV = p.R / (p.gamma - 1.0);
    // Compute_P_from_U in FP64 (base_shll.c:171-176 / base_shll_2d.c:312-318)
    for (size_t c = 0; c < n; c++) {
        double u0 = U[c];
        double p1 = U[n + c] / u0;
        if (nv == 3) {
            if (rho) rho[c] = u0;
            if (u) u[c] = p1;
            if (T) T[c] = ((U[2 * n + c] / u0) - 0.5 * p1 * p1) / CV;
        } else {
            double p2 = U[2 * n + c] / u0;
            if (rho) rho[c] = u0;
            if (u) u[c] = p1;
            if (v) v[c] = p2;
            if (T) T[c] = ((U[3 * n + c] / u0) - 0.5 * (p1 * p1 + p2 * p2)) / CV;
        }
    }
    return SHLL_OK;
}

int mixed_get_primitives(MixedState* m, double* rho, double* u, double* v, double* T, char* err, size_t len) {
    return mixed_item_primitives(m, 0, rho, u, v, T, err, len);
}
int mixed_get_conserved(MixedState* m, double* planes, char* err, size_t len) {
    return mixed_item_conserved(m, 0, planes, err, len);
}

int mixed_item_totals(MixedState* m, int item, double* out, char* err, size_t len) {
    if (item < 0 || item >= m->nitems) { snprintf(err, len, "item %d out of range", item); return SHLL_ERR_ARG; }
    if (m->dim == 2) return mixed2d_totals(m, item, out, err, len);
    const TubeP& tp = m->tubes[item];
    const int b = m->par[item];
    double tmp[3];
    for (int k = 0; k < 3; k++) {
        const size_t off = (size_t)k * m->plane + tp.base;
        cudaError_t e = m->kahan
            ? device_pair_sums(static_cast<float*>(m->hi[b]) + off, m->lo[b] + off, 1, tp.n, &tmp[k], m->stream)
            : device_plane_sums(static_cast<double*>(m->hi[b]) + off, 64, 1, tp.n, &tmp[k], m->stream);
        if (e != cudaSuccess) { snprintf(err, len, "totals failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    }
    for (int k = 0; k < 3; k++) out[k] = tmp[k];
    return SHLL_OK;
}

int mixed_totals(MixedState* m, double* out, char* err, size_t len) { return mixed_item_totals(m, 0, out, err, len); }

// accessors used by mixed2d.cu
cudaStream_t mixed_stream(MixedState* m) { return m->stream; }
int* mixed_flag_ptr(MixedState* m) { return m->d_flag; }
int* mixed_item_flags_ptr(MixedState* m) { return m->d_item_flags; }

int mixed_item_flags(MixedState* m, int item) {
    if (item < 0 || item >= m->nitems || !m->d_item_flags) return 0;
    int h = 0;
    cudaMemcpyAsync(&h, m->d_item_flags + item, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
    cudaStreamSynchronize(m->stream);
    return h;
}
const shll_params* mixed_items(MixedState* m, int* count) { *count = m->nitems; return m->items.data(); }
void** mixed_d2_slot(MixedState* m) { return &m->d2; }
int mixed_fold(MixedState* m) { return m->B; }
bool mixed_is_kahan(MixedState* m) { return m->kahan; }
void mixed_add_updates(MixedState* m, long u) { m->cell_updates += u; }

// copies both state buffers (the buffer a tube lives in differs per tube) and the parities
int mixed_checkpoint(MixedState* m, bool restore, char* err, size_t len) {
    if (m->dim == 2) { snprintf(err, len, "checkpoint of 2D mixed state not supported"); return SHLL_ERR_UNSUPPORTED; }
    const size_t vb = (size_t)m->plane * 3 * (m->kahan ? sizeof(float) : sizeof(double));
    const size_t lb = (size_t)m->plane * 3 * sizeof(float);
    if (restore && !m->ck_hi[0]) { snprintf(err, len, "no checkpoint taken"); return SHLL_ERR_STATE; }
    for (int b = 0; b < 2; b++) {
        if (!restore && !m->ck_hi[b]) {
            if (cudaMalloc(&m->ck_hi[b], vb) != cudaSuccess || (m->kahan && cudaMalloc(&m->ck_lo[b], lb) != cudaSuccess)) {
                snprintf(err, len, "checkpoint allocation failed");
                return SHLL_ERR_NOMEM;
            }
        }
        cudaError_t e = restore ? cudaMemcpyAsync(m->hi[b], m->ck_hi[b], vb, cudaMemcpyDeviceToDevice, m->stream)
                                : cudaMemcpyAsync(m->ck_hi[b], m->hi[b], vb, cudaMemcpyDeviceToDevice, m->stream);
        if (e == cudaSuccess && m->kahan)
            e = restore ? cudaMemcpyAsync(m->lo[b], m->ck_lo[b], lb, cudaMemcpyDeviceToDevice, m->stream)
                        : cudaMemcpyAsync(m->ck_lo[b], m->lo[b], lb, cudaMemcpyDeviceToDevice, m->stream);
        if (e != cudaSuccess) { snprintf(err, len, "checkpoint copy failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    }
    if (restore) { m->par = m->ck_par; m->cell_updates = m->ck_updates; }
    else { m->ck_par = m->par; m->ck_updates = m->cell_updates; }
    return SHLL_OK;
}

// ------------------------------------------------------------------------------------------
// Entry point for callers that cannot allocate device memory.
//
// Some host programs cannot call cudaMalloc at the point where they want to advance a tube: an
// allocator that the process has reserved or capped for itself, a real-time loop that must not
// take the allocator's locks, or a host that hands the library device buffers it manages
// itself.  shll_tube_run_static() advances one 1D tube held in the caller's device buffer with
// the same sweep kernels as the context API, and keeps everything else it needs (the second
// state buffer, the boundary flux sums, the chunk descriptors and the error flag) in the
// fixed array below.  That array is part of the library image: every GPU that loads the library
// holds its 2 MiB until the process exits.
namespace {
constexpr int kStaticMaxCells = 65536;                 // largest tube the static scratch can hold
constexpr int kStaticMaxChunks = 256;
constexpr size_t kStaticStateBytes = (size_t)3 * kStaticMaxCells * sizeof(double);
constexpr size_t kStaticBSumOff = kStaticStateBytes;                                  // 2 x BSum[256]
constexpr size_t kStaticChunkOff = kStaticBSumOff + 2 * kStaticMaxChunks * sizeof(BSum);
constexpr size_t kStaticTubeOff = (kStaticChunkOff + kStaticMaxChunks * sizeof(Chunk) + 255) / 256 * 256;
constexpr size_t kStaticFlagOff = kStaticTubeOff + 256;
constexpr size_t kStaticScratchBytes = 2u << 20;
static_assert(kStaticFlagOff + 256 <= kStaticScratchBytes, "static scratch layout exceeds its array");
constexpr int kStaticMaxDevices = 64;
}  // namespace

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

static std::mutex g_static_mu;
static void* g_static_addr[kStaticMaxDevices];  // device address of g_static_scratch, per device

// The device address of the scratch array on the current device, looked up once per device.
// The host-side name g_static_scratch is only a stand-in: a kernel must be given this address.
static int static_scratch(void** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kStaticMaxDevices) {
        fprintf(stderr, "shll_tube_run_static: no usable current device (%s)\n", cudaGetErrorString(e));
        return SHLL_ERR_CUDA;
    }
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_addr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_static_scratch);
        if (e != cudaSuccess || !p) {
            fprintf(stderr, "shll_tube_run_static: cudaGetSymbolAddress failed on device %d: %s\n", dev,
                    cudaGetErrorString(e));
            return SHLL_ERR_CUDA;
        }
        g_static_addr[dev] = p;
    }
    *out = g_static_addr[dev];
    return SHLL_OK;
}

extern "C" int shll_tube_run_static(const shll_params* p, double* d_cons, long nsteps, void* stream) {
    if (!p || !d_cons) {
        fprintf(stderr, "shll_tube_run_static: params and state buffer are required\n");
        return SHLL_ERR_ARG;
    }
    if (p->dim != 1 || (p->order != 1 && p->order != 2) || p->precision != SHLL_PREC_MIXED_F64) {
        fprintf(stderr, "shll_tube_run_static: takes one 1D tube (order 1 or 2) in SHLL_PREC_MIXED_F64\n");
        return SHLL_ERR_ARG;
    }
    if (p->nx < 2 || p->nx > kStaticMaxCells) {
        fprintf(stderr, "shll_tube_run_static: %d cells is outside 2..%d, the size of the static scratch\n", p->nx,
                kStaticMaxCells);
        return SHLL_ERR_ARG;
    }
    if (reinterpret_cast<uintptr_t>(d_cons) % alignof(double) != 0) {
        fprintf(stderr, "shll_tube_run_static: state buffer is not 8-byte aligned\n");
        return SHLL_ERR_ARG;
    }
    if (nsteps <= 0) nsteps = shll_steps_for(p);
    if (nsteps <= 0 || nsteps > (1L << 30)) {
        fprintf(stderr, "shll_tube_run_static: invalid step count\n");
        return SHLL_ERR_ARG;
    }
    void* base = nullptr;
    int rc = static_scratch(&base);
    if (rc != SHLL_OK) return rc;
    unsigned char* sc = static_cast<unsigned char*>(base);
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // descriptors of the tube, built on the stack
    const int fold = p->fold_steps > 0 ? p->fold_steps : 16;
    const int B = std::min(fold, MW / 16);
    TubeP tp;
    memset(&tp, 0, sizeof(tp));
    tp.base = 0;
    tp.n = p->nx;
    tp.order = p->order;
    tp.limiter = p->limiter;
    tp.gamma = p->gamma;
    tp.R = p->R;
    double lamy;
    item_consts(*p, &tp.CV, &tp.lam, &lamy);
    tp.alpha = (float)p->mc_alpha;
    {
        int ex;
        tp.lam_pow2 = std::frexp(tp.lam, &ex) == 0.5 && ex > -100 && ex < 100;
    }
    tp.steps = (int)nsteps;
    tp.par = 0;
    Chunk chunks[kStaticMaxChunks];
    const int n = tp.n;
    const int S = chunk_owned(tp.order, B);
    int k = n <= MW ? 2 : (n + S - 1) / S;
    if (k > n) k = n;
    if (k > kStaticMaxChunks) {
        fprintf(stderr, "shll_tube_run_static: %d chunks exceed the static limit %d\n", k, kStaticMaxChunks);
        return SHLL_ERR_ARG;
    }
    for (int c = 0; c < k; c++) {
        const int a = (int)((long)n * c / k), b = (int)((long)n * (c + 1) / k);
        const int anc = c == 0 ? 0 : (c == k - 1 ? n - 1 : (a + b) / 2);
        chunks[c] = {0, a, b, anc, c, c > 0 ? c - 1 : -1, c + 1 < k ? c + 1 : -1};
    }
    TubeP* d_tube = reinterpret_cast<TubeP*>(sc + kStaticTubeOff);
    Chunk* d_chunks = reinterpret_cast<Chunk*>(sc + kStaticChunkOff);
    int* d_flag = reinterpret_cast<int*>(sc + kStaticFlagOff);
    cudaError_t e = cudaMemcpyAsync(d_tube, &tp, sizeof(tp), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_chunks, chunks, sizeof(Chunk) * k, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_flag, 0, sizeof(int), s);  // the flag must start clear
    if (e != cudaSuccess) {
        fprintf(stderr, "shll_tube_run_static: descriptor upload failed: %s\n", cudaGetErrorString(e));
        return SHLL_ERR_CUDA;
    }
    SweepArgs A;
    A.tubes = d_tube;
    A.chunks = d_chunks;
    A.hi[0] = d_cons;
    A.hi[1] = sc;  // the second state buffer
    A.lo[0] = A.lo[1] = nullptr;
    A.bsum[0] = reinterpret_cast<BSum*>(sc + kStaticBSumOff);
    A.bsum[1] = A.bsum[0] + kStaticMaxChunks;
    A.plane = n;
    A.B = B;
    A.flag = d_flag;
    A.item_flags = nullptr;
    const long nsweeps = (nsteps + B - 1) / B;
    shll_count_launches(nsweeps + 1);
    for (long w = 0; w < nsweeps; w++) {
        A.sweep = (int)w;
        k_sweep1d<false><<<k, MT, 0, s>>>(A);
    }
    k_fixup1d<false><<<(k + 127) / 128, 128, 0, s>>>(A, k);
    e = cudaGetLastError();
    if (e == cudaSuccess && (nsweeps & 1))  // the result ended in the scratch buffer: copy it back
        e = cudaMemcpyAsync(d_cons, sc, (size_t)3 * n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, d_flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        fprintf(stderr, "shll_tube_run_static: %s\n", cudaGetErrorString(e));
        return SHLL_ERR_CUDA;
    }
    if (flag & SHLL_FLAG_BADARG) return SHLL_ERR_ARG;
    if (flag & SHLL_FLAG_NONPOSITIVE) return SHLL_ERR_NUMERIC;
    return SHLL_OK;
}

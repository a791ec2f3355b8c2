// Mixed-precision 1D SHLL engine: FP32 split fluxes in perturbation form, compensated FP32
// accumulation, FP64 (or FP32-pair) state folded once per fold window of sweeps.
//
// Scheme (the arithmetic of base-c/base_shll.c:87-159 and of the x sweep of
// base-c/2nd_order_base_shll.c:203-459, re-associated as interface fluxes):
//   * Cells are grouped in chunks (one CTA each).  A chunk is computed over a window of its own
//     cells plus a halo of order*steps cells on each side (temporal blocking), so a sweep
//     advances every chunk of every tube by B steps with no exchange inside it; a chunk's next
//     sweep needs only its two neighbours' previous one.  Runs that fit on the GPU at once are one
//     resident launch in which each chunk waits for its neighbours (k_tube1d); larger ones are
//     one launch per sweep (k_sweep1d).
//   * Every chunk has one frame: the FP64 state U* of an anchor cell at the start of the window
//     (the wall cell for the first and last chunk of a tube, else the centre cell) and the
//     split-flux coefficients derived from it.  Each window cell's split fluxes are evaluated in
//     FP32 as deviations from the frame (d fp = fp(U) - fp(U*), d fm likewise), with only
//     deviations as FP32 operands, so their rounding error scales with |U - U*| instead of |U|.
//   * The flux through interface j+1/2 is Fref + Delta_{j+1/2} (Fref = the anchor's physical
//     flux, which cancels inside a chunk); both neighbouring cells add the same FP32 value
//     lam*Delta with opposite signs (TwoSum into an FP32 value+compensation pair per cell).
//   * Neighbouring chunks evaluate their shared boundary interface in different frames, so the
//     two values differ by rounding.  Each chunk records the flux it applied at both of its
//     boundaries over the sweep; at the end of the next sweep the right chunk's first cell
//     receives lam*sum(F_left chunk - F_right chunk) (a fix-up kernel applies the last sweep's
//     after a run), which makes the left chunk's value the one that counts: mass, momentum and
//     energy are conserved to the rounding of the FP64 state.  Applied at the end, the correction
//     is not needed before a sweep's first step, and the copies of a cell in two windows stay
//     identical (both see the stored value).
//   * At the end of a sweep the pair is added to the stored state: in FP64
//     (SHLL_PREC_MIXED_F64) or in FP32-pair arithmetic (SHLL_PREC_MIXED_KAHAN).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "mixed.h"
#include "mixed_common.cuh"
#include "shll_internal.h"

namespace {

constexpr int MW = 512;       // window capacity (cells) of one CTA
constexpr int MT = MW / 2;    // threads per CTA: two adjacent cells per thread (FP32x2 lanes)
constexpr int kSweepSteps = 16;      // steps per sweep (temporal blocking depth)
constexpr int kDefaultFold1D = 64;   // default FP64 fold interval (steps), 1D
constexpr int kDefaultFold2D = 64;   // 2D

struct TubeP {
    long base;        // offset of cell 0 in the planes
    int n, order, limiter;
    int steps;        // steps of the current run
    int par;          // buffer holding the tube's state at the start of the run
    double gamma, R, CV, lam;
    double RoCV;      // R / CV: P = (R/CV) (E - m u / 2)
    float alpha;
    float gRf, Rf, cvinvf;  // gamma R, R, 1/CV in FP32
    int lam_pow2;     // lam is a power of two: lam*Delta is exact in FP32
    int B;            // steps per sweep (temporal blocking depth, <= MW / 16)
    int fold_sweeps;  // sweeps per fold window (FP64 state read at the first, written at the last)
    int owned;        // owned cells per chunk (0: the window minus the halos)
    float gg1p[2], gm1p[2];  // gamma (gamma-1) and gamma-1 = R/CV as FP32 pairs (pair flux)
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

// Frame of an anchor state.  FP64 only where the frame's values enter the state directly: the
// anchor flux F (boundary-flux sums, walls) and, for first-order wall chunks, the wall split
// fluxes fpS1/fmS1.  1/rho and 1/a come from FP32 seeds refined by Newton steps in FP64
// (r <- r (2 - rho r) doubles the correct bits: 2^-22 -> 2^-44 -> 2^-88).  The FP32
// coefficients only multiply deviations, so FP32 accuracy suffices for them.  Run by one thread:
// every FP64 operation costs a full warp slot of the narrow FP64 pipe, so their number is kept
// small (about 15, plus 15 for wall chunks of first order).
__device__ void make_frame(Frame1& f, const double U[3], const TubeP& tp, bool wall_fluxes) {
    const double rho = U[0], m = U[1], E = U[2];
    double r = f2d_bits(fast_rcp(d2f_bits(rho)));
    r = fma(r, fma(-rho, r, 1.0), r);
    r = fma(r, fma(-rho, r, 1.0), r);
    const double u0 = m * r;
    const double u = fma(r, fma(-rho, u0, m), u0);
    const double P = tp.RoCV * fma(-0.5 * m, u, E);
    const double F[3] = {m, fma(m, u, P), u * (E + P)};
    for (int k = 0; k < 3; k++) {
        f.U[k] = U[k];
        f.F[k] = F[k];
        f.c.F[k] = d2f_bits(F[k]);
        d2ff_bits(U[k], f.Uh[k], f.Ul[k]);
        f.c.Uf[k] = f.Uh[k];
    }
    const float rf = d2f_bits(r), uf = d2f_bits(u), Pf = d2f_bits(P);
    const float Tf = __fmul_rn(__fmul_rn(Pf, rf), fast_rcp(tp.Rf));
    const float a2 = __fmul_rn(tp.gRf, Tf);
    const float ainv = rsqrtf(a2);
    const float af = __fmul_rn(a2, ainv);
    const float Mf = __fmul_rn(uf, ainv);
    f.c.rho = d2f_bits(rho); f.c.u = uf; f.c.v = 0.f; f.c.e = __fmul_rn(f.c.Uf[2], rf); f.c.T = Tf;
    f.c.a = af; f.c.M = Mf; f.c.P = Pf; f.c.Z1 = __fmul_rn(0.5f, __fadd_rn(Mf, 1.0f));
    f.c.Z2 = __fmul_rn(__fmul_rn(0.5f, af), __fmaf_rn(-Mf, Mf, 1.0f));
    f.c.gR = tp.gRf; f.c.R = tp.Rf; f.c.cvinv = tp.cvinvf;
    f.fpS1 = f.fmS1 = 0.0;
    if (wall_fluxes) {  // a^2 = gamma P / rho; y = 1/a by Newton steps y <- y (3/2 - a^2 y^2 / 2)
        const double A2 = tp.gamma * P * r;
        double y = f2d_bits(rsqrtf(d2f_bits(A2)));
        const double h = 0.5 * A2;
        y = y * fma(-h * y, y, 1.5);
        y = y * fma(-h * y, y, 1.5);
        const double a = A2 * y, M = u * y;
        const double Z1 = fma(0.5, M, 0.5), Z3 = Z1 - 1.0, Z2 = 0.5 * a * fma(-M, M, 1.0);
        f.fpS1 = fma(F[1], Z1, m * Z2);
        f.fmS1 = -fma(F[1], Z3, m * Z2);
    }
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
    float* dh[2];       // deviation pairs between the sweeps of a fold window (value, compensation)
    float* dl[2];
    Frame1* frames;     // per chunk id: the frame of the current fold window
    long plane;         // cells per plane (all tubes)
    int sweep;
    int chunk0;         // first chunk of the launch (chunks are grouped by scheme variant)
    int* flag;
    int* item_flags;    // per tube (may be null)
    int stall_id;       // resident runs, test hook: this chunk never publishes its progress (-1: none)
    // first order: per chunk id and sweep parity, 1 if an owned cell's Mach number exceeded
    // kPairMach at the end of that sweep; a chunk's sweep uses the pair flux when it or a
    // neighbour had one at the end of the previous sweep.  Null: FP32 flux throughout.
    int* mode[2];
    float pair_m2;      // the squared Mach number that sets a flag (negative: every chunk, a test hook)
};

// Mach number above which a first-order chunk and its neighbours evaluate their fluxes in
// double-FP32 arithmetic (the reference scheme amplifies rounding errors where M > 1; the margin
// also covers cells that accelerate past M = 1 during the next sweep, and subsonic cells whose
// FP32 rounding errors the flow carries into the supersonic region)
constexpr float kPairMach = 0.6f;
// dynamic shared memory of a pair-flux sweep: the remainders of the split fluxes
constexpr int kPairSmem = 2 * 2 * 3 * MW * (int)sizeof(float);

// the pair-flux decision for a chunk's sweep `sweep` (flags of the previous sweep, or of the
// state at the start of the run for sweep 0); L2 loads, as the flags are written by other blocks
__device__ __forceinline__ bool pair_mode(const SweepArgs& A, const Chunk& ch, int sweep) {
    const int* f = ((sweep - 1) & 1) ? A.mode[1] : A.mode[0];
    int v = __ldcg(f + ch.id);
    if (ch.idL >= 0) v |= __ldcg(f + ch.idL);
    if (ch.idR >= 0) v |= __ldcg(f + ch.idR);
    return v != 0;
}

// correction owed to the first owned cell of the chunk with id `right` by its left neighbour
// `left` for the sweep whose sums are in bs: lam*sum(F_left) - lam*sum(F_right) at their interface
__device__ __forceinline__ double boundary_correction(const BSum* bs, int left, int right, int k) {
    return bs[left].s[1][k] - bs[right].s[0][k];
}

struct Smem1 {
    Frame1 fr;
    alignas(16) float sfp[2][3][MW];    // split-flux deviations, double-buffered by step parity
    alignas(16) float sfm[2][3][MW];
    float wall[2][3][2];                // constant wall terms (order 1) for cell 0 / n-1
    float corrp[3][2];                  // correction owed to cell a by the previous sweep, FP32 pairs
    float dnb[2][3][2];                 // U*(left / right neighbour) - U*(this chunk), FP32 pairs
    float rec[2][MW / 16][3][2];        // per-step terms at the chunk's boundary interfaces
};
constexpr int kFrameWords = (int)(sizeof(Frame1) / 4);
static_assert(sizeof(Frame1) % 4 == 0 && kFrameWords <= MT, "frame copy by one word per thread");


// loads of values written by other blocks: from L2 (ld.global.cg) in the resident kernel, where
// this SM's L1 may still hold lines of an earlier sweep of the same launch
template <bool CG, class T>
__device__ __forceinline__ T ldx(const T* p) {
    if (CG) return __ldcg(p);
    return *p;
}

// One sweep of one chunk.  Thread t holds window cells w0 = 2t and w0 + 1 as the two lanes of
// FP32x2 registers.  Per step: split-flux deviations of both cells (packed) -> shared memory
// (buffer of the step's parity) -> one barrier -> the thread evaluates the three interfaces
// w0-1/2, w0+1/2, w0+3/2 that its cells need (the outer two are also evaluated, bit for bit
// identically, by the neighbouring threads) -> TwoSum accumulation of lam*(F_in - F_out).
// The double buffer makes the second barrier of a store/load/store pattern unnecessary: a
// thread can only overwrite a buffer after every thread has passed the barrier that follows
// the last reads of it.
// FF: first order only, the split fluxes, interface sums and accumulation in double-FP32
// arithmetic (flux1x2_ff); a launch of either form leaves the chunks whose pair-flux decision
// (pair_mode) calls for the other form to the other launch of the same sweep.
// RES: called by the resident kernel (k_tube1d), which keeps the frame and the neighbour-frame
// offsets in shared memory for a whole fold window.  reuse: the owned cells' deviation pairs are
// taken from dh/dl (this thread's registers after the previous sweep of the same geometry)
// instead of memory; keep: the next sweep will do so, so only the cells that the neighbours read
// as halo are stored.
template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM, bool RES, bool FF = false>
__device__ void sweep_chunk(const SweepArgs& A, const int sweep, const Chunk& ch, const TubeP& tp, Smem1& S,
                            float2 (&dh)[3], float2 (&dl)[3], const bool reuse, const bool keep) {
    constexpr int R_ = ORDER;  // stencil reach per step
    Frame1& fr = S.fr;

    const int tid = threadIdx.x;
    const int n = tp.n;
    const int steps = min(tp.B, tp.steps - sweep * tp.B);
    if (steps <= 0) return;
    const int H = R_ * steps;
    const int ws = max(0, ch.a - H), we = min(n, ch.b + H), L = we - ws;
    const int pa = ch.a - ws, pb = ch.b - ws;  // first owned / one past the last owned, window coords
    const int inb = (tp.par + sweep) & 1, outb = inb ^ 1;
    // position in the fold window: the first sweep reads the stored state and sets the frame,
    // the last one writes the state back; the sweeps between exchange deviation pairs
    const int F = tp.fold_sweeps;
    const int jw = sweep % F;
    const int nsw = (tp.steps + tp.B - 1) / tp.B;
    const bool wstart = jw == 0;
    const bool wend = jw == F - 1 || sweep == nsw - 1;
    // frames of this window written two or more launches ago may be read before the wait (see
    // k_sweep1d); L2-only loads, as this SM's L1 may hold the previous window's lines
    const bool early = !RES && !wstart && jw >= 2;
    unsigned fw = 0;
    double va = 0.0, vb = 0.0;   // threads 0-5: a correction va - vb; 6-11: a frame offset va - vb
    if (early) {
        if (tid < kFrameWords) fw = __ldcg(reinterpret_cast<const unsigned*>(&A.frames[ch.id]) + tid);
        if (tid >= 6 && tid < 12) {
            const int side = (tid % 6) / 3, k = tid % 3;
            const int nb = side == 0 ? ch.idL : ch.idR;
            if (nb >= 0) { va = __ldcg(&A.frames[nb].U[k]); vb = __ldcg(&A.frames[ch.id].U[k]); }
        }
    }
    if (!RES) {
        asm volatile("griddepcontrol.wait;" ::: "memory");
        asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
        // (block-uniform: every thread reads the same flags)
        if (A.mode[0] && pair_mode(A, ch, sweep) != FF) return;
    }
    // (selects rather than indexing the parameter arrays, which would copy them to local memory)
    const void* hin = inb ? A.hi[1] : A.hi[0];
    const float* lin = inb ? A.lo[1] : A.lo[0];
    const float* dhin = inb ? A.dh[1] : A.dh[0];
    const float* dlin = inb ? A.dl[1] : A.dl[0];
    const long base = tp.base;
    const long P = A.plane;
    const double lam = tp.lam;
    const float lamh = (float)lam, laml = (float)(lam - (double)lamh);

    if (L > MW || tp.B > MW / 16 || tp.B < 1) {  // host guarantees this never happens; refuse rather than overrun
        if (tid == 0) atomicOr(A.flag, SHLL_FLAG_BADARG);
        return;
    }
    // the window's stored values, loaded first so that their latency overlaps the frame setup
    const int w0 = 2 * tid;
    double uin[2][3];           // FP64 state (window start)
    float uh[2][3], ul[2][3];   // FP32 value + compensation (KAHAN window start), or deviation pair
#pragma unroll
    for (int q = 0; q < 2; q++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            uin[q][k] = 0.0; uh[q][k] = 0.f; ul[q][k] = 0.f;
            const int w = w0 + q;
            if (w < L) {
                const long idx = k * P + base + ws + w;
                if (!wstart) {
                    if (reuse && w >= pa && w < pb) { uh[q][k] = lane(dh[k], q); ul[q][k] = lane(dl[k], q); }
                    else { uh[q][k] = ldx<RES>(dhin + idx); ul[q][k] = ldx<RES>(dlin + idx); }
                } else if (KAHAN) {
                    uh[q][k] = ldx<RES>(static_cast<const float*>(hin) + idx);
                    ul[q][k] = ldx<RES>(lin + idx);
                } else {
                    uin[q][k] = ldx<RES>(static_cast<const double*>(hin) + idx);
                }
            }
        }
    // The frame: computed from the anchor cell at the start of a fold window (one thread), copied
    // from the per-chunk table by the other sweeps of the window (one word per thread); either way
    // it is in shared memory after the barrier below
    const Frame1* frp = &fr;
    // every load of this prologue is issued before any of its values is used: a shared-memory
    // store of a loaded value stalls the warp until that load returns (in-order issue), which
    // would serialise the L2 round trips
    if (!RES && !wstart && !early && tid < kFrameWords) fw = reinterpret_cast<const unsigned*>(&A.frames[ch.id])[tid];
    // threads 0-2: the correction owed to cell a by the previous sweep, lam*sum(F_left - F_right)
    // at the interface a-1/2 (the left neighbour's record minus this chunk's), which the owner of
    // cell a adds at the end of this sweep; threads 6-11: the neighbour-frame offsets
    const bool cthread = tid < 3 || (tid >= 6 && tid < 12 && !wstart && (!RES || jw == 1));
    if (cthread) {
        const int side = (tid % 6) / 3, k = tid % 3;
        if (tid < 3) {
            if (sweep > 0 && ch.idL >= 0) {
                const BSum* bs = ((sweep - 1) & 1) ? A.bsum[1] : A.bsum[0];
                va = ldx<RES>(&bs[ch.idL].s[1][k]);
                vb = ldx<RES>(&bs[ch.id].s[0][k]);
            }
        } else if (!early) {
            const int nb = side == 0 ? ch.idL : ch.idR;
            if (nb >= 0) { va = ldx<RES>(&A.frames[nb].U[k]); vb = ldx<RES>(&A.frames[ch.id].U[k]); }
        }
    }
    if (!RES && !wstart && tid < kFrameWords) reinterpret_cast<unsigned*>(&fr)[tid] = fw;
    // as FP32 pairs, once per block; the resident kernel converts the correction only after the
    // steps, so that its loads do not hold up the first step
    if (cthread && !(RES && tid < 3)) {
        const int side = (tid % 6) / 3, k = tid % 3;
        float* o = tid < 3 ? S.corrp[k] : S.dnb[side][k];
        d2ff_bits(va - vb, o[0], o[1]);
    }
    if (wstart) {
        if (tid == 0) {
            double U[3];
            float Uanc_h[3], Uanc_l[3];
            for (int k = 0; k < 3; k++) {
                const long idx = k * P + base + ch.anc;
                if (KAHAN) {
                    Uanc_h[k] = ldx<RES>(static_cast<const float*>(hin) + idx);
                    Uanc_l[k] = ldx<RES>(lin + idx);
                    U[k] = f2d_bits(Uanc_h[k]) + f2d_bits(Uanc_l[k]);
                } else {
                    U[k] = ldx<RES>(static_cast<const double*>(hin) + idx);
                }
            }
            make_frame(fr, U, tp, ORDER == 1 && (ch.idL < 0 || ch.idR < 0));
            if (KAHAN)  // the stored pair itself, so that the anchor cell's deviation is exactly 0
                for (int k = 0; k < 3; k++) { fr.Uh[k] = Uanc_h[k]; fr.Ul[k] = Uanc_l[k]; }
        }
    }
    // (a resident sweep inside a window after its second writes no shared memory before its first
    // step: frame and neighbour offsets are kept, the correction is converted later)
    if (!RES || jw < 2) __syncthreads();
    if (wstart && !wend && tid < kFrameWords)  // keep the frame for the rest of the window
        reinterpret_cast<unsigned*>(&A.frames[ch.id])[tid] = reinterpret_cast<const unsigned*>(&fr)[tid];
    if (tid < 6 && ORDER == 1) {
        // reflective walls: constant parts of the wall-cell increments (read after the first step's
        // barrier)
        // cell 0:   lam*F_{-1/2} - lam*Fref = (-lam F0, lam (2 fmS1 - F1), -lam F2) (+2 lam dfm1_0)
        // cell n-1: lam*Fref - lam*F_{n-1/2} = (lam F0, lam (F1 - 2 fpS1), lam F2) (-2 lam dfp1_{n-1})
        const int bnd = tid / 3, k = tid % 3;
        double w = bnd == 0 ? (k == 1 ? lam * (2.0 * frp->fmS1 - frp->F[1]) : -lam * frp->F[k])
                            : (k == 1 ? lam * (frp->F[1] - 2.0 * frp->fpS1) : lam * frp->F[k]);
        d2ff_bits(w, S.wall[bnd][k][0], S.wall[bnd][k][1]);
    }

    // ---- the window as deviations from the frame ----
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int w = w0 + q;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            float h = 0.f, l = 0.f;
            if (w < L) {
                if (!wstart) {
                    // deviation pair relative to the owner's frame -> relative to this frame
                    h = uh[q][k]; l = ul[q][k];
                    if (w < pa || w >= pb) {
                        const int sd = w < pa ? 0 : 1;
                        ff_add(h, l, S.dnb[sd][k][0], S.dnb[sd][k][1], h, l);
                    }
                } else {
                    if (KAHAN) ff_sub(uh[q][k], ul[q][k], frp->Uh[k], frp->Ul[k], h, l);
                    else d2ff_bits(uin[q][k] - frp->U[k], h, l);
                }
            }
            set_lane(dh[k], q, h);
            set_lane(dl[k], q, l);
        }
    }
    const Coef2 c2 = coef2(frp->c);
    const bool hasL = ch.idL >= 0, hasR = ch.idR >= 0;
    // loop-invariant roles of this thread's cells (i = tube cell of window cell w)
    auto edge = [&](int w) { const int i = ws + w; return i <= 0 || i >= n - 1; };
    // half-slope factors: 0.5, or 0 on edge cells (the reference's zero slopes there) and on the
    // ghost cells beyond the walls
    const float2 hp = make_float2(edge(w0) ? 0.f : 0.5f, edge(w0 + 1) ? 0.f : 0.5f);
    const float2 nhm = neg2(hp);
    const float hpl = edge(w0 - 1) ? 0.f : 0.5f;    // cell w0 - 1 (sp only)
    const float nhmr = edge(w0 + 2) ? -0.f : -0.5f; // cell w0 + 2 (sm only)
    // Second order (outflow walls, base-c/2nd_order_base_shll.c:236-262): the wall flux is the
    // cell's own flux fp + fm, i.e. the regular interface formula with a ghost cell that copies
    // the wall cell (fp_{-1} = fp_0, fm_n = fm_{n-1}, zero slopes), so walls need no special
    // path.  The ghost values are substituted by selects in the wall threads.
    const bool gl = ORDER == 2 && ws + w0 == 0;            // lane x is cell 0
    const bool grx = ORDER == 2 && ws + w0 == n - 1;       // lane x is cell n-1
    const bool gry = ORDER == 2 && ws + w0 + 1 == n - 1;   // lane y is cell n-1
    // interface masks: a cell's left / right interface is applied unless it lies outside the
    // window or (first order) is a reflective wall, whose flux the wall terms supply
    auto in_ok = [&](int w) {
        const int i = ws + w;
        if (w >= L) return false;
        return ORDER == 2 ? (w > 0 || i == 0) : (i > 0 && w > 0);
    };
    auto out_ok = [&](int w) {
        const int i = ws + w;
        if (w >= L) return false;
        return ORDER == 2 ? (w < L - 1 || i == n - 1) : (i < n - 1 && w < L - 1);
    };
    // lam per lane and side, 0 where the interface is not applied (the mask folded into lam)
    const float2 lin2 = make_float2(in_ok(w0) ? lamh : 0.f, in_ok(w0 + 1) ? lamh : 0.f);
    const float2 lout2 = make_float2(out_ok(w0) ? lamh : 0.f, out_ok(w0 + 1) ? lamh : 0.f);
    const float2 llin2 = make_float2(in_ok(w0) ? laml : 0.f, in_ok(w0 + 1) ? laml : 0.f);
    const float2 llout2 = make_float2(out_ok(w0) ? laml : 0.f, out_ok(w0 + 1) ? laml : 0.f);
    // first-order reflective walls: lane q is cell 0 or n-1 (a few threads)
    bool wallq[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int w = w0 + q, i = ws + w;
        wallq[q] = ORDER == 1 && w < L && (i == 0 || i == n - 1);
    }
    const bool any_wall = wallq[0] || wallq[1];
    // chunk-boundary records: the terms applied at interface a-1/2 (cell a's left) and b-1/2
    // (cell b-1's right) are stored per step and summed at the end of the sweep
    const bool rin0 = hasL && w0 == pa, rin1 = hasL && w0 + 1 == pa;
    const bool rout0 = hasR && w0 == pb - 1, rout1 = hasR && w0 + 1 == pb - 1;
    const bool any_rec = rin0 || rin1 || rout0 || rout1;
    const int jl = max(w0 - 2, 0), jr = min(w0 + 2, MW - 2);  // neighbour pairs (clamped)

    if constexpr (FF) {
        // The same step in double-FP32 arithmetic: each cell's state U = U* + (dh + dl) as a pair,
        // its physical split fluxes as pairs (values in S.sfp / S.sfm, remainders in dynamic
        // shared memory), and the increment lam (F_{j-1/2} - F_{j+1/2}) of the full interface fluxes
        // added to the deviation pair with a renormalising sum.  Reflective walls (first order):
        // the wall flux (0, 2 fm1_0, 0) at cell 0 and (0, 2 fp1_{n-1}, 0) at cell n-1
        // (base-c/base_shll.c:93-110); the boundary records keep the FP32 form's meaning,
        // lam (F - Fref).
        extern __shared__ __align__(16) float g_pair_smem[];
        float* sfpl = g_pair_smem;               // [2][3][MW]
        float* sfml = g_pair_smem + 2 * 3 * MW;  // [2][3][MW]
        auto at = [](float* base, int b, int k, int w) { return reinterpret_cast<float2*>(base + (b * 3 + k) * MW + w); };
        const FF2 gg1 = ffv(tp.gg1p[0], tp.gg1p[1]), gm1 = ffv(tp.gm1p[0], tp.gm1p[1]);
        for (int s = 0; s < steps; s++) {
            const int b = s & 1;
            FF2 fp[3], fm[3];
            {
                FF2 U[3];
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    const FF2 d = ffnorm(dh[k], dl[k]);
                    dh[k] = d.h;
                    dl[k] = d.l;
                    U[k] = ffadd(ffv(frp->Uh[k], frp->Ul[k]), d);
                }
                flux1x2_ff(U, gg1, gm1, fp, fm);
            }
#pragma unroll
            for (int k = 0; k < 3; k++) {
                if (grx) {  // ghost fm_n of the right outflow wall (lane y holds no cell)
                    fm[k].h.y = fm[k].h.x;
                    fm[k].l.y = fm[k].l.x;
                }
                *reinterpret_cast<float2*>(&S.sfp[b][k][w0]) = fp[k].h;
                *reinterpret_cast<float2*>(&S.sfm[b][k][w0]) = fm[k].h;
                *at(sfpl, b, k, w0) = fp[k].l;
                *at(sfml, b, k, w0) = fm[k].l;
            }
            __syncthreads();
#pragma unroll
            for (int k = 0; k < 3; k++) {
                const FF2 pL = {*reinterpret_cast<const float2*>(&S.sfp[b][k][jl]), *at(sfpl, b, k, jl)};  // fp_{w0-2}, fp_{w0-1}
                const FF2 mR = {*reinterpret_cast<const float2*>(&S.sfm[b][k][jr]), *at(sfml, b, k, jr)};  // fm_{w0+2}, fm_{w0+3}
                FF2 IN, OUT;
                if constexpr (ORDER == 1) {
                    IN = ffadd_u({make_float2(pL.h.y, fp[k].h.x), make_float2(pL.l.y, fp[k].l.x)}, fm[k]);
                    OUT = ffadd_u(fp[k], {make_float2(fm[k].h.y, mR.h.x), make_float2(fm[k].l.y, mR.l.x)});
                } else {  // the FP32 step's reconstruction (see below), in pairs
                    const FF2 pR = {*reinterpret_cast<const float2*>(&S.sfp[b][k][jr]), *at(sfpl, b, k, jr)};  // fp_{w0+2}
                    const FF2 mL = {*reinterpret_cast<const float2*>(&S.sfm[b][k][jl]), *at(sfml, b, k, jl)};  // fm_{w0-1}
                    // fp_{w0-1} (ghost of the left wall: fp_0) and fm_{w0+2} (ghost of the right wall: fm_{n-1})
                    const float fplh = gl ? fp[k].h.x : pL.h.y, fpll = gl ? fp[k].l.x : pL.l.y;
                    const float fmrh = gry ? fm[k].h.y : mR.h.x, fmrl = gry ? fm[k].l.y : mR.l.x;
                    // differences f_j - f_{j-1}
                    const FF2 dpo = ffsub(fp[k], {make_float2(fplh, fp[k].h.x), make_float2(fpll, fp[k].l.x)});  // j = w0, w0+1
                    const FF2 dpr = ffsub({make_float2(fp[k].h.y, pR.h.x), make_float2(fp[k].l.y, pR.l.x)}, fp[k]);  // j = w0+1, w0+2
                    const FF2 dmo = ffsub(fm[k], {make_float2(mL.h.y, fm[k].h.x), make_float2(mL.l.y, fm[k].l.x)});
                    const FF2 dmr = ffsub({make_float2(fm[k].h.y, fmrh), make_float2(fm[k].l.y, fmrl)}, fm[k]);
                    // lane x: fp_{w0-1} - fp_{w0-2}; lane y: fm_{w0+3} - fm_{w0+2}
                    const FF2 dedge = ffsub({make_float2(fplh, mR.h.y), make_float2(fpll, mR.l.y)},
                                            {make_float2(pL.h.x, fmrh), make_float2(pL.l.x, fmrl)});
                    const FF2 sp = ffslope<LIM>(dpo, dpr, tp.alpha), sm = ffslope<LIM>(dmo, dmr, tp.alpha);
                    // lane x: the slope of fp at w0-1; lane y: the slope of fm at w0+2
                    const FF2 se = ffslope<LIM>({make_float2(dedge.h.x, dmr.h.y), make_float2(dedge.l.x, dmr.l.y)},
                                                {make_float2(dpo.h.x, dedge.h.y), make_float2(dpo.l.x, dedge.l.y)}, tp.alpha);
                    // reconstructed L_j = fp_j + sp_j/2 and R_j = fm_j - sm_j/2 (factors 0 on edge cells: exact)
                    const FF2 Lo = ffadd(fp[k], {mul2(hp, sp.h), mul2(hp, sp.l)});
                    const FF2 Ro = ffadd(fm[k], {mul2(nhm, sm.h), mul2(nhm, sm.l)});
                    const float2 fe = make_float2(hpl, nhmr);
                    const FF2 Le = ffadd({make_float2(fplh, fmrh), make_float2(fpll, fmrl)}, {mul2(fe, se.h), mul2(fe, se.l)});
                    IN = ffadd_u({make_float2(Le.h.x, Lo.h.x), make_float2(Le.l.x, Lo.l.x)}, Ro);
                    OUT = ffadd_u(Lo, {make_float2(Ro.h.y, Le.h.y), make_float2(Ro.l.y, Le.l.y)});
                }
                FF2 tin, tout;
                if (LAM_POW2) {  // lam a power of two (or 0 where masked): exact scaling
                    tin = {mul2(lin2, IN.h), mul2(lin2, IN.l)};
                    tout = {mul2(lout2, OUT.h), mul2(lout2, OUT.l)};
                } else {
                    tin = ffmul_u(IN, {lin2, llin2});
                    tout = ffmul_u(OUT, {lout2, llout2});
                }
                FF2 v = ffadd({dh[k], dl[k]}, ffsub(tin, tout));
                if (any_wall && k == 1) {  // (the wall's own interface is masked out of tin / tout)
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        if (!wallq[q]) continue;
                        const bool left = ws + w0 + q == 0;
                        const float sg = left ? 2.f : -2.f;  // + lam 2 fm1 at cell 0, - lam 2 fp1 at cell n-1
                        const FF2 wf = {f2(sg * lane(left ? fm[1].h : fp[1].h, q)), f2(sg * lane(left ? fm[1].l : fp[1].l, q))};
                        const FF2 t = LAM_POW2 ? ffscale(wf, lamh) : ffmul_u(wf, ffv(lamh, laml));
                        const FF2 vq = ffadd({f2(lane(v.h, q)), f2(lane(v.l, q))}, t);
                        set_lane(v.h, q, vq.h.x);
                        set_lane(v.l, q, vq.l.x);
                    }
                }
                dh[k] = v.h;
                dl[k] = v.l;
                if (any_rec) {  // lam (F - Fref) at the chunk's boundary interfaces
                    float fh, fl;
                    d2ff_bits(frp->F[k], fh, fl);
                    const FF2 lref = LAM_POW2 ? ffscale(ffv(fh, fl), lamh) : ffmul(ffv(fh, fl), ffv(lamh, laml));
                    const FF2 ri = ffsub(tin, lref), ro = ffsub(tout, lref);
                    if (rin0) { S.rec[0][s][k][0] = ri.h.x; S.rec[0][s][k][1] = ri.l.x; }
                    if (rin1) { S.rec[0][s][k][0] = ri.h.y; S.rec[0][s][k][1] = ri.l.y; }
                    if (rout0) { S.rec[1][s][k][0] = ro.h.x; S.rec[1][s][k][1] = ro.l.x; }
                    if (rout1) { S.rec[1][s][k][0] = ro.h.y; S.rec[1][s][k][1] = ro.l.y; }
                }
            }
        }
    } else
    for (int s = 0; s < steps; s++) {
        const int b = s & 1;
        // ---- split-flux deviations of both cells ----
        float2 fp[3], fm[3];
        {
            float2 d[3];
#pragma unroll
            for (int k = 0; k < 3; k++) d[k] = add2(dh[k], dl[k]);
            dflux1x2(c2, d, fp, fm);
        }
#pragma unroll
        for (int k = 0; k < 3; k++) {
            if (grx) fm[k].y = fm[k].x;  // ghost fm_n of the right wall (lane y holds no cell)
            *reinterpret_cast<float2*>(&S.sfp[b][k][w0]) = fp[k];
            *reinterpret_cast<float2*>(&S.sfm[b][k][w0]) = fm[k];
        }
        __syncthreads();
        // ---- interfaces w0-1/2 (IN.x), w0+1/2 (IN.y = OUT.x), w0+3/2 (OUT.y) ----
        float2 ihk[3], ohk[3], ilk[3], olk[3];  // applied terms (for the boundary records)
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const float2 pL = *reinterpret_cast<const float2*>(&S.sfp[b][k][jl]);  // fp_{w0-2}, fp_{w0-1}
            const float2 mR = *reinterpret_cast<const float2*>(&S.sfm[b][k][jr]);  // fm_{w0+2}, fm_{w0+3}
            float2 IN, OUT;
            if (ORDER == 1) {
                IN = add2(make_float2(pL.y, fp[k].x), fm[k]);
                OUT = add2(fp[k], make_float2(fm[k].y, mR.x));
            } else {
                const float2 pR = *reinterpret_cast<const float2*>(&S.sfp[b][k][jr]);  // fp_{w0+2}
                const float2 mL = *reinterpret_cast<const float2*>(&S.sfm[b][k][jl]);  // fm_{w0-1}
                const float fpl = gl ? fp[k].x : pL.y;    // fp_{w0-1} (ghost of the left wall)
                const float fmr = gry ? fm[k].y : mR.x;   // fm_{w0+2} (ghost of the right wall)
                // differences f_j - f_{j-1}
                const float2 dpo = sub2(fp[k], make_float2(fpl, fp[k].x));      // j = w0, w0+1
                const float2 dpr = sub2(make_float2(fp[k].y, pR.x), fp[k]);     // j = w0+1, w0+2
                const float dpl = __fadd_rn(fpl, -pL.x);                         // j = w0-1
                const float2 dmo = sub2(fm[k], make_float2(mL.y, fm[k].x));
                const float2 dmr = sub2(make_float2(fm[k].y, fmr), fm[k]);
                const float dmrr = __fadd_rn(mR.y, -fmr);                        // j = w0+3
                // reconstructed left states L_j = fp_j + sp_j/2 and right states R_j = fm_j - sm_j/2
                const float2 Lo = fma2(hp, slope2<LIM>(dpo, dpr, tp.alpha), fp[k]);           // j = w0, w0+1
                const float Ll = __fmaf_rn(hpl, slope_s<LIM>(dpl, dpo.x, tp.alpha), fpl);       // j = w0-1
                const float2 Ro = fma2(nhm, slope2<LIM>(dmo, dmr, tp.alpha), fm[k]);          // j = w0, w0+1
                const float Rr = __fmaf_rn(nhmr, slope_s<LIM>(dmr.y, dmrr, tp.alpha), fmr);     // j = w0+2
                IN = add2(make_float2(Ll, Lo.x), Ro);
                OUT = add2(Lo, make_float2(Ro.y, Rr));
            }
            const float2 ih = mul2(lin2, IN), oh = mul2(lout2, OUT);
            float2 il = f2(0.f), ol = f2(0.f);
            if (!LAM_POW2) {
                il = add2(fma2(lin2, IN, neg2(ih)), mul2(llin2, IN));
                ol = add2(fma2(lout2, OUT, neg2(oh)), mul2(llout2, OUT));
            }
            two_sum_acc2(dh[k], dl[k], ih);
            two_diff_acc2(dh[k], dl[k], oh);
            if (!LAM_POW2) dl[k] = add2(dl[k], sub2(il, ol));
            ihk[k] = ih; ohk[k] = oh; ilk[k] = il; olk[k] = ol;
        }
        if (any_rec) {  // the threads of cells a and b-1 (warp-uniform elsewhere)
#pragma unroll
            for (int k = 0; k < 3; k++) {
                if (rin0) { S.rec[0][s][k][0] = ihk[k].x; S.rec[0][s][k][1] = ilk[k].x; }
                if (rin1) { S.rec[0][s][k][0] = ihk[k].y; S.rec[0][s][k][1] = ilk[k].y; }
                if (rout0) { S.rec[1][s][k][0] = ohk[k].x; S.rec[1][s][k][1] = olk[k].x; }
                if (rout1) { S.rec[1][s][k][0] = ohk[k].y; S.rec[1][s][k][1] = olk[k].y; }
            }
        }
        // ---- first-order reflective walls (the threads of cells 0 and n-1) ----
        if (ORDER == 1 && any_wall) {
#pragma unroll
            for (int q = 0; q < 2; q++) {
                if (!wallq[q]) continue;
                const int i = ws + w0 + q;
                const int bnd = i == 0 ? 0 : 1;
#pragma unroll
                for (int k = 0; k < 3; k++) {
                    float h = lane(dh[k], q), l = lane(dl[k], q);
                    two_sum_acc(h, l, S.wall[bnd][k][0]); l = __fadd_rn(l, S.wall[bnd][k][1]);
                    if (k == 1) {  // +2 lam dfm1_0 at the left wall, -2 lam dfp1_{n-1} at the right
                        const float v = i == 0 ? __fmul_rn(2.f, lane(fm[1], q)) : -__fmul_rn(2.f, lane(fp[1], q));
                        const float vh = __fmul_rn(lamh, v);
                        const float vl = __fadd_rn(__fmaf_rn(lamh, v, -vh), __fmul_rn(laml, v));
                        two_sum_acc(h, l, vh); l = __fadd_rn(l, vl);
                    }
                    set_lane(dh[k], q, h);
                    set_lane(dl[k], q, l);
                }
            }
        }
    }
    if (RES && tid < 3) d2ff_bits(va - vb, S.corrp[tid][0], S.corrp[tid][1]);   // (read after the barrier)
    // ---- boundary flux sums of this sweep (full flux: steps * lam * Fref + sum lam*Delta) ----
    __syncthreads();
    if (tid < 6) {
        const int side = tid / 3, k = tid % 3;
        if (side == 0 ? hasL : hasR) {
            float h = 0.f, l = 0.f;
            for (int st = 0; st < steps; st++) {
                two_sum_acc(h, l, S.rec[side][st][k][0]);
                l = __fadd_rn(l, S.rec[side][st][k][1]);
            }
            BSum* bout = ((sweep & 1) ? A.bsum[1] : A.bsum[0]) + ch.id;
            bout->s[side][k] = steps * lam * frp->F[k] + (f2d_bits(h) + f2d_bits(l));
        }
    }

    // ---- fold the owned cells into the stored state (last sweep of a window), or pass their
    // deviation pairs to the next sweep ----
    int bad = 0;
    int fast = 0;   // an owned cell above the pair-flux Mach number (first order)
    void* hout = outb ? A.hi[1] : A.hi[0];
    float* lout = outb ? A.lo[1] : A.lo[0];
    float* dhout = outb ? A.dh[1] : A.dh[0];
    float* dlout = outb ? A.dl[1] : A.dl[0];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int w = w0 + q;
        if (w < pa || w >= pb) continue;
        float uf[3];
        bool finite = true;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            const long idx = k * P + base + ws + w;
            float h = lane(dh[k], q), l = lane(dl[k], q);
            if (w == pa && hasL && sweep > 0) {  // the previous sweep's correction of cell a
                ff_add(h, l, S.corrp[k][0], S.corrp[k][1], h, l);
                set_lane(dh[k], q, h);
                set_lane(dl[k], q, l);
            }
            finite = finite && isfinite(h) && isfinite(l);
            if (!wend) {
                if (!keep || w < pa + H || w >= pb - H) {  // (keep: only the neighbours' halo cells)
                    dhout[idx] = h;
                    dlout[idx] = l;
                }
                uf[k] = __fadd_rn(frp->Uh[k], h);
            } else if (KAHAN) {
                float oh, ol;
                ff_add(frp->Uh[k], frp->Ul[k], h, l, oh, ol);
                static_cast<float*>(hout)[idx] = oh;
                lout[idx] = ol;
                uf[k] = oh;
            } else {
                static_cast<double*>(hout)[idx] = frp->U[k] + (f2d_bits(h) + f2d_bits(l));
                uf[k] = __fadd_rn(frp->Uh[k], h);  // FP32 estimate, for the positivity check only
            }
        }
        const float eint = __fadd_rn(uf[2], -__fmul_rn(0.5f, __fdividef(__fmul_rn(uf[1], uf[1]), uf[0])));
        // breakdown: non-positive density or internal energy, or an overflowed / NaN increment
        bad |= !(uf[0] > 0.f) || !(eint > 0.f) || !finite;
        // M^2 = m^2 / (rho^2 a^2) with a^2 = gamma (gamma-1) eint / rho (second order: the pair flux
        // only where it is asked for everywhere)
        if (ORDER == 1)
            fast |= __fmul_rn(uf[1], uf[1]) >
                    __fmul_rn(A.pair_m2, __fmul_rn(__fmul_rn(tp.gRf, tp.cvinvf), __fmul_rn(uf[0], eint)));
        else
            fast |= A.pair_m2 < 0.f;
    }
    if (bad) {
        atomicOr(A.flag, SHLL_FLAG_NONPOSITIVE);
        if (A.item_flags) atomicOr(&A.item_flags[ch.tube], SHLL_FLAG_NONPOSITIVE);
    }
    if (A.mode[0]) {
        const int any = __syncthreads_or(fast);
        if (tid == 0) ((sweep & 1) ? A.mode[1] : A.mode[0])[ch.id] = any;
    }
}

// One specialised kernel per scheme variant keeps each kernel's code small (the step loop is
// latency-bound with few warps per SM, so instruction-fetch bubbles show directly).
// Consecutive sweeps are chained by programmatic dependent launch: once a sweep has passed its
// own griddepcontrol.wait it lets the next one launch (griddepcontrol.launch_dependents); the next
// sweep's blocks become resident beside it, read what does not depend on it (descriptors, and
// frames written two or more launches earlier) and wait in griddepcontrol.wait until this grid
// has completed and its memory is visible (a hardware dependency, no polling).
template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM>
__global__ void __launch_bounds__(MT, 3) k_sweep1d(SweepArgs A) {
    __shared__ Smem1 S;
    const Chunk ch = A.chunks[A.chunk0 + blockIdx.x];
    const TubeP tp = A.tubes[ch.tube];
    float2 dh[3], dl[3];
    // (waits for the previous sweep inside)
    sweep_chunk<ORDER, KAHAN, LAM_POW2, LIM, false>(A, A.sweep, ch, tp, S, dh, dl, false, false);
}

// The pair-flux form of a first-order sweep, launched after the FP32 form for the same chunks
// (each block runs its chunk only when the chunk's pair-flux decision calls for it).  Its own
// kernel so that the longer double-FP32 step does not raise the register count, and so lower the
// occupancy, of the FP32 sweeps.
template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM>
__global__ void __launch_bounds__(MT, 2) k_sweep1d_ff(SweepArgs A) {
    __shared__ Smem1 S;
    const Chunk ch = A.chunks[A.chunk0 + blockIdx.x];
    const TubeP tp = A.tubes[ch.tube];
    float2 dh[3], dl[3];
    sweep_chunk<ORDER, KAHAN, LAM_POW2, LIM, false, true>(A, A.sweep, ch, tp, S, dh, dl, false, false);
}

// The pair-flux flags of the state at the start of a run (as sweep -1 would leave them): one block
// per chunk.  A chunk is flagged when an owned cell exceeds the Mach threshold or when the
// pressure within kJumpReach cells of its cells varies by more than the factor kPairJump: a gas at
// rest at a diaphragm has M = 0, but the first sweep already accelerates it, and the FP32 rounding
// of that sweep would be carried into the supersonic region that forms there.
constexpr float kPairJump = 1.5f;
constexpr int kJumpReach = 16;
template <bool KAHAN>
__global__ void __launch_bounds__(256) k_mode1d(SweepArgs A) {
    __shared__ float wmax[8], wmin[8];
    const Chunk ch = A.chunks[blockIdx.x];
    const TubeP tp = A.tubes[ch.tube];
    int fast = tp.order == 2 && A.pair_m2 < 0.f;   // second order: only where asked for everywhere
    float pmax = 0.f, pmin = 3.0e38f;
    if (tp.order == 1) {
        const void* hin = tp.par ? A.hi[1] : A.hi[0];
        const float* lin = tp.par ? A.lo[1] : A.lo[0];
        const double g = tp.gamma * (tp.gamma - 1.0);
        const int lo = max(0, ch.a - kJumpReach), hi = min(tp.n, ch.b + kJumpReach);
        for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
            const long idx = tp.base + i;
            const double r = load_state<KAHAN>(hin, lin, idx);
            const double m = load_state<KAHAN>(hin, lin, A.plane + idx);
            const double E = load_state<KAHAN>(hin, lin, 2 * A.plane + idx);
            const double eint = E - 0.5 * m * m / r;
            if (i >= ch.a && i < ch.b) fast |= m * m > (double)A.pair_m2 * g * r * eint;
            const float P = (float)(tp.RoCV * eint);
            pmax = fmaxf(pmax, P);
            pmin = fminf(pmin, P);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        pmax = fmaxf(pmax, __shfl_xor_sync(0xffffffffu, pmax, o));
        pmin = fminf(pmin, __shfl_xor_sync(0xffffffffu, pmin, o));
    }
    if ((threadIdx.x & 31) == 0) { wmax[threadIdx.x >> 5] = pmax; wmin[threadIdx.x >> 5] = pmin; }
    fast = __syncthreads_or(fast);
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) { pmax = fmaxf(pmax, wmax[w]); pmin = fminf(pmin, wmin[w]); }
        A.mode[1][ch.id] = fast || (tp.order == 1 && pmax > kPairJump * pmin);
    }
}

// polls of the neighbours' progress counters before a resident block gives up (under a second,
// at about half a microsecond per poll; a sweep of a co-resident neighbour takes tens of
// microseconds)
constexpr long kSpinLimit = 1L << 20;
// progress counters one 128-byte line apart: a poll then touches only the counter's own line, so
// the pollers of one chunk do not delay the release stores of the others
constexpr int kProgStride = 32;

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_gpu(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// The resident form of a run: one block per chunk for all sweeps of the run (a cooperative
// launch, so every block is resident at once).  A chunk's sweep k needs only the previous sweep
// of its two neighbours (their halo cells, boundary sums and frames), so instead of one launch
// per sweep each block waits for its neighbours' progress counters (prog[id] = sweeps completed,
// published with release semantics after the block's stores).  The frame and the neighbour-frame
// offsets stay in shared memory for a whole fold window, and the owned cells' deviation pairs stay
// in registers between the sweeps of a window that have the same geometry; only the cells within
// the halo width of a chunk edge go through memory.  Write-after-read is covered by the same
// counters: the buffer that sweep k + 1 writes was read by the neighbours' sweep k, which has
// completed.  Each wait is bounded: a block that gives up sets SHLL_FLAG_TIMEOUT and returns, and
// so, bounded again, do the blocks waiting for it.
// FM: the flux arithmetic, 0 FP32 (no pair-flux code in the kernel), 1 chosen per chunk and sweep
// by the pair-flux flags (first order), 2 double-FP32 in every sweep (the pair flux everywhere).
// CLU: the cluster form (k_cluster1d): the chunks of one tube are one thread-block cluster, and the
// wait between sweeps is the cluster's hardware barrier (release / acquire at cluster scope) instead
// of the neighbours' progress counters; the data still goes through L2.
template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM, int FM, bool CLU>
__device__ __forceinline__ void tube_run(const SweepArgs& A, unsigned* prog) {
    __shared__ Smem1 S;
    __shared__ int s_ok;
    const Chunk ch = A.chunks[A.chunk0 + blockIdx.x];
    const TubeP tp = A.tubes[ch.tube];
    const int nsw = (tp.steps + tp.B - 1) / tp.B;
    const int F = tp.fold_sweeps;
    float2 dh[3], dl[3];
    for (int sw = 0; sw < nsw; sw++) {
        if (CLU && sw > 0) {
            // every block of the cluster (every chunk of the tube) has completed the previous sweep
            asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
        } else if (sw > 0) {
            if (threadIdx.x == 0) {
                // both counters polled at once (a chunk without a neighbour on one side reads its
                // own counter there, which is ahead)
                const unsigned* pl = prog + (long)(ch.idL >= 0 ? ch.idL : ch.id) * kProgStride;
                const unsigned* pr = prog + (long)(ch.idR >= 0 ? ch.idR : ch.id) * kProgStride;
                bool ok = false;
                for (long it = 0; it < kSpinLimit && !ok; it++) {
                    const unsigned vl = ld_acquire_gpu(pl), vr = ld_acquire_gpu(pr);
                    ok = vl >= (unsigned)sw && vr >= (unsigned)sw;
                    if (!ok) {
                        // another block gave up: so does this one (now rather than after its own
                        // limit; every 64th poll, as all blocks read this word)
                        if ((it & 63) == 63 && (ld_acquire_gpu(reinterpret_cast<const unsigned*>(A.flag)) & SHLL_FLAG_TIMEOUT))
                            break;
                        __nanosleep(32);
                    }
                }
                if (!ok) atomicOr(A.flag, SHLL_FLAG_TIMEOUT);
                s_ok = ok;
            }
            __syncthreads();
            if (!s_ok) return;
        }
        // sweeps of B steps inside a fold window share the geometry of the one before
        const bool reuse = sw % F != 0 && tp.steps - sw * tp.B >= tp.B;
        const bool keep = sw + 1 < nsw && (sw + 1) % F != 0 && tp.steps - (sw + 1) * tp.B >= tp.B;
        // (FM 1: the neighbours' flags of the previous sweep are visible after the wait above, as
        // they were written before the neighbours' release; block-uniform)
        if constexpr (FM == 2)
            sweep_chunk<ORDER, KAHAN, LAM_POW2, LIM, true, true>(A, sw, ch, tp, S, dh, dl, reuse, keep);
        else if (FM == 1 && A.mode[0] && pair_mode(A, ch, sw))
            sweep_chunk<ORDER, KAHAN, LAM_POW2, LIM, true, FM == 1>(A, sw, ch, tp, S, dh, dl, reuse, keep);
        else
            sweep_chunk<ORDER, KAHAN, LAM_POW2, LIM, true>(A, sw, ch, tp, S, dh, dl, reuse, keep);
        __syncthreads();
        // (the barrier orders the block's stores before thread 0's release at GPU scope)
        if (!CLU && threadIdx.x == 0 && ch.id != A.stall_id)
            st_release_gpu(prog + (long)ch.id * kProgStride, (unsigned)(sw + 1));
    }
}

template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM, int FM>
__global__ void __launch_bounds__(MT, 1) k_tube1d(SweepArgs A, unsigned* prog) {
    tube_run<ORDER, KAHAN, LAM_POW2, LIM, FM, false>(A, prog);
}

// The cluster form of a resident run (launched with one cluster per tube, all tubes of the launch
// with the same number of chunks, at most 16): no grid-wide residency needed, each tube advances
// on its own.
template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM, int FM>
__global__ void __launch_bounds__(MT, 1) k_cluster1d(SweepArgs A) {
    tube_run<ORDER, KAHAN, LAM_POW2, LIM, FM, true>(A, nullptr);
}

// scheme variant of a tube: 0/1 first order (lam a power of two or not), 2/3 second order
// minmod, 4/5 second order MC limiter
static int tube_variant(const TubeP& tp) {
    if (tp.order == 1) return tp.lam_pow2 ? 0 : 1;
    return 2 + (tp.limiter == 1 ? 2 : 0) + (tp.lam_pow2 ? 0 : 1);
}

// multiprocessors of the current device (cached per device)
static int device_sms() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
    if (cache[dev] == 0) {
        int v = 1;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 1;
    }
    return cache[dev];
}

// Dynamic shared memory that keeps a sweep block alone on its SM.  For a grid of at most one
// block per SM the next sweep's blocks (launched early, see k_sweep1d) could otherwise be packed
// two or three to an SM while others stay empty; with this padding each one waits for an SM of
// its own.  Grids of several waves launch without it.
constexpr int kSoloSmem = 120 * 1024;

template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM>
static cudaError_t launch_one(int grid, cudaStream_t s, const SweepArgs& A, bool pdl) {
    static unsigned long long attr_set = 0;  // devices on which the padding is allowed
    int dev = 0;
    cudaGetDevice(&dev);
    const bool solo = pdl && grid <= device_sms();
    if (solo && dev < 64 && !(attr_set & (1ull << dev))) {
        cudaError_t e = cudaFuncSetAttribute(k_sweep1d<ORDER, KAHAN, LAM_POW2, LIM>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, kSoloSmem);
        if (e != cudaSuccess) return e;
        attr_set |= 1ull << dev;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(MT);
    cfg.dynamicSmemBytes = solo ? kSoloSmem : 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_sweep1d<ORDER, KAHAN, LAM_POW2, LIM>, A);
}

// allows the padding on every variant kernel of the current device (before any stream capture)
static cudaError_t allow_solo_padding() {
    static unsigned long long done = 0;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev >= 64 || (done & (1ull << dev))) return e;
    const void* ks[] = {
        (const void*)k_sweep1d<1, false, true, 0>, (const void*)k_sweep1d<1, true, true, 0>,
        (const void*)k_sweep1d<1, false, false, 0>, (const void*)k_sweep1d<1, true, false, 0>,
        (const void*)k_sweep1d<2, false, true, 0>, (const void*)k_sweep1d<2, true, true, 0>,
        (const void*)k_sweep1d<2, false, false, 0>, (const void*)k_sweep1d<2, true, false, 0>,
        (const void*)k_sweep1d<2, false, true, 1>, (const void*)k_sweep1d<2, true, true, 1>,
        (const void*)k_sweep1d<2, false, false, 1>, (const void*)k_sweep1d<2, true, false, 1>,
        (const void*)k_sweep1d_ff<1, false, true, 0>, (const void*)k_sweep1d_ff<1, true, true, 0>,
        (const void*)k_sweep1d_ff<1, false, false, 0>, (const void*)k_sweep1d_ff<1, true, false, 0>,
        (const void*)k_sweep1d_ff<2, false, true, 0>, (const void*)k_sweep1d_ff<2, true, true, 0>,
        (const void*)k_sweep1d_ff<2, false, false, 0>, (const void*)k_sweep1d_ff<2, true, false, 0>,
        (const void*)k_sweep1d_ff<2, false, true, 1>, (const void*)k_sweep1d_ff<2, true, true, 1>,
        (const void*)k_sweep1d_ff<2, false, false, 1>, (const void*)k_sweep1d_ff<2, true, false, 1>};
    for (const void* k : ks) {
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kSoloSmem);
        if (e != cudaSuccess) return e;
    }
    done |= 1ull << dev;
    return cudaSuccess;
}

// pdl: chain to the previous sweep of the same run (the first sweep of a run follows the
// descriptor uploads with ordinary stream order)
static cudaError_t launch_sweep(int variant, bool kahan, int grid, cudaStream_t s, const SweepArgs& A, bool pdl) {
    switch (variant * 2 + (kahan ? 1 : 0)) {
        case 0: return launch_one<1, false, true, 0>(grid, s, A, pdl);
        case 1: return launch_one<1, true, true, 0>(grid, s, A, pdl);
        case 2: return launch_one<1, false, false, 0>(grid, s, A, pdl);
        case 3: return launch_one<1, true, false, 0>(grid, s, A, pdl);
        case 4: return launch_one<2, false, true, 0>(grid, s, A, pdl);
        case 5: return launch_one<2, true, true, 0>(grid, s, A, pdl);
        case 6: return launch_one<2, false, false, 0>(grid, s, A, pdl);
        case 7: return launch_one<2, true, false, 0>(grid, s, A, pdl);
        case 8: return launch_one<2, false, true, 1>(grid, s, A, pdl);
        case 9: return launch_one<2, true, true, 1>(grid, s, A, pdl);
        case 10: return launch_one<2, false, false, 1>(grid, s, A, pdl);
        default: return launch_one<2, true, false, 1>(grid, s, A, pdl);
    }
}

// the pair-flux sweep of a first-order variant group (variants 0, 1); its dynamic shared memory
// holds the remainders of the split fluxes (within the padding when the grid is a single wave)
template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM>
static cudaError_t launch_one_ff(int grid, cudaStream_t s, const SweepArgs& A, bool pdl) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(MT);
    cfg.dynamicSmemBytes = pdl && grid <= device_sms() ? kSoloSmem : kPairSmem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k_sweep1d_ff<ORDER, KAHAN, LAM_POW2, LIM>, A);
}
static cudaError_t launch_sweep_ff(int variant, bool kahan, int grid, cudaStream_t s, const SweepArgs& A, bool pdl) {
    switch (variant * 2 + (kahan ? 1 : 0)) {
        case 0: return launch_one_ff<1, false, true, 0>(grid, s, A, pdl);
        case 1: return launch_one_ff<1, true, true, 0>(grid, s, A, pdl);
        case 2: return launch_one_ff<1, false, false, 0>(grid, s, A, pdl);
        case 3: return launch_one_ff<1, true, false, 0>(grid, s, A, pdl);
        case 4: return launch_one_ff<2, false, true, 0>(grid, s, A, pdl);
        case 5: return launch_one_ff<2, true, true, 0>(grid, s, A, pdl);
        case 6: return launch_one_ff<2, false, false, 0>(grid, s, A, pdl);
        case 7: return launch_one_ff<2, true, false, 0>(grid, s, A, pdl);
        case 8: return launch_one_ff<2, false, true, 1>(grid, s, A, pdl);
        case 9: return launch_one_ff<2, true, true, 1>(grid, s, A, pdl);
        case 10: return launch_one_ff<2, false, false, 1>(grid, s, A, pdl);
        default: return launch_one_ff<2, true, false, 1>(grid, s, A, pdl);
    }
}
static_assert(kPairSmem <= kSoloSmem, "the pair-flux buffers fit in the padding of single-wave sweeps");

// resident form of a run (k_tube1d): a cooperative launch of one block per chunk, each alone on
// its SM (the same shared-memory padding as single-wave sweeps)
template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM, int FM>
static cudaError_t launch_res(int grid, cudaStream_t s, const SweepArgs& A, unsigned* prog, bool check_only) {
    static unsigned long long attr_set = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !(attr_set & (1ull << dev))) {
        cudaError_t e = cudaFuncSetAttribute(k_tube1d<ORDER, KAHAN, LAM_POW2, LIM, FM>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, kSoloSmem);
        if (e != cudaSuccess) return e;
        attr_set |= 1ull << dev;
    }
    if (check_only) {  // every block must be resident at once
        int per_sm = 0;
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tube1d<ORDER, KAHAN, LAM_POW2, LIM, FM>,
                                                                      MT, kSoloSmem);
        if (e != cudaSuccess) return e;
        return (long)per_sm * device_sms() >= grid ? cudaSuccess : cudaErrorCooperativeLaunchTooLarge;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(MT);
    cfg.dynamicSmemBytes = kSoloSmem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeCooperative;
    at[0].val.cooperative = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_tube1d<ORDER, KAHAN, LAM_POW2, LIM, FM>, A, prog);
}

// cluster form: grid = the run's chunks, clusters of `csize` consecutive chunks (one tube each)
template <int ORDER, bool KAHAN, bool LAM_POW2, int LIM, int FM>
static cudaError_t launch_clu(int grid, int csize, cudaStream_t s, const SweepArgs& A, bool check_only) {
    static unsigned long long attr_set = 0;
    int dev = 0;
    cudaGetDevice(&dev);
    auto* kern = k_cluster1d<ORDER, KAHAN, LAM_POW2, LIM, FM>;
    if (dev < 64 && !(attr_set & (1ull << dev))) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSoloSmem);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        if (e != cudaSuccess) return e;
        attr_set |= 1ull << dev;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(MT);
    cfg.dynamicSmemBytes = kSoloSmem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)csize;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    if (check_only) {   // at least one cluster of this size fits the GPU
        int n = 0;
        cudaError_t e = cudaOccupancyMaxActiveClusters(&n, kern, &cfg);
        if (e != cudaSuccess) return e;
        return n >= 1 ? cudaSuccess : cudaErrorInvalidConfiguration;
    }
    return cudaLaunchKernelEx(&cfg, kern, A);
}

static cudaError_t launch_cluster(int variant, bool kahan, int grid, int csize, cudaStream_t s, const SweepArgs& A,
                                  bool check_only) {
    switch (variant * 2 + (kahan ? 1 : 0)) {
        case 0: return launch_clu<1, false, true, 0, 1>(grid, csize, s, A, check_only);
        case 1: return launch_clu<1, true, true, 0, 1>(grid, csize, s, A, check_only);
        case 2: return launch_clu<1, false, false, 0, 1>(grid, csize, s, A, check_only);
        case 3: return launch_clu<1, true, false, 0, 1>(grid, csize, s, A, check_only);
        case 4: return launch_clu<2, false, true, 0, 0>(grid, csize, s, A, check_only);
        case 5: return launch_clu<2, true, true, 0, 0>(grid, csize, s, A, check_only);
        case 6: return launch_clu<2, false, false, 0, 0>(grid, csize, s, A, check_only);
        case 7: return launch_clu<2, true, false, 0, 0>(grid, csize, s, A, check_only);
        case 8: return launch_clu<2, false, true, 1, 0>(grid, csize, s, A, check_only);
        case 9: return launch_clu<2, true, true, 1, 0>(grid, csize, s, A, check_only);
        case 10: return launch_clu<2, false, false, 1, 0>(grid, csize, s, A, check_only);
        default: return launch_clu<2, true, false, 1, 0>(grid, csize, s, A, check_only);
    }
}

// all_pairs: the pair flux everywhere (second order then needs the pair-flux kernel; first order
// chooses per chunk and sweep either way)
static cudaError_t launch_resident(int variant, bool kahan, int grid, cudaStream_t s, const SweepArgs& A,
                                   unsigned* prog, bool check_only, bool all_pairs) {
    const int v = variant * 2 + (kahan ? 1 : 0);
    if (variant >= 2 && all_pairs) {
        switch (v) {
            case 4: return launch_res<2, false, true, 0, 2>(grid, s, A, prog, check_only);
            case 5: return launch_res<2, true, true, 0, 2>(grid, s, A, prog, check_only);
            case 6: return launch_res<2, false, false, 0, 2>(grid, s, A, prog, check_only);
            case 7: return launch_res<2, true, false, 0, 2>(grid, s, A, prog, check_only);
            case 8: return launch_res<2, false, true, 1, 2>(grid, s, A, prog, check_only);
            case 9: return launch_res<2, true, true, 1, 2>(grid, s, A, prog, check_only);
            case 10: return launch_res<2, false, false, 1, 2>(grid, s, A, prog, check_only);
            default: return launch_res<2, true, false, 1, 2>(grid, s, A, prog, check_only);
        }
    }
    switch (v) {
        case 0: return launch_res<1, false, true, 0, 1>(grid, s, A, prog, check_only);
        case 1: return launch_res<1, true, true, 0, 1>(grid, s, A, prog, check_only);
        case 2: return launch_res<1, false, false, 0, 1>(grid, s, A, prog, check_only);
        case 3: return launch_res<1, true, false, 0, 1>(grid, s, A, prog, check_only);
        case 4: return launch_res<2, false, true, 0, 0>(grid, s, A, prog, check_only);
        case 5: return launch_res<2, true, true, 0, 0>(grid, s, A, prog, check_only);
        case 6: return launch_res<2, false, false, 0, 0>(grid, s, A, prog, check_only);
        case 7: return launch_res<2, true, false, 0, 0>(grid, s, A, prog, check_only);
        case 8: return launch_res<2, false, true, 1, 0>(grid, s, A, prog, check_only);
        case 9: return launch_res<2, true, true, 1, 0>(grid, s, A, prog, check_only);
        case 10: return launch_res<2, false, false, 1, 0>(grid, s, A, prog, check_only);
        default: return launch_res<2, true, false, 1, 0>(grid, s, A, prog, check_only);
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
    const int sweeps = (tp.steps + tp.B - 1) / tp.B;
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
    float* dh[2] = {nullptr, nullptr};   // deviation pairs between the sweeps of a fold window
    float* dl[2] = {nullptr, nullptr};
    Frame1* frames = nullptr;            // per chunk: frame of the current fold window
    int* mode[2] = {nullptr, nullptr};   // per chunk, by sweep parity: pair-flux flags
    bool has_first = false;              // a first-order tube (the only ones flagged by default)
    unsigned* prog = nullptr;            // per chunk: sweeps completed in a resident run
    size_t prog_n = 0;
    double* stage = nullptr;             // device staging of one item's primitive planes
    size_t stage_words = 0;
    int* d_bad = nullptr;                // first non-positive cell of an upload
    int* d_bad_items = nullptr;          // the same per item (uploads of every item at once)
    // captured launch sequences of earlier runs, replayed when a run repeats (same step counts and
    // buffer parities)
    struct GraphEntry {
        std::vector<long> steps;
        std::vector<int> par;
        cudaGraphExec_t exec;
        long launches;
    };
    std::vector<GraphEntry> graphs;
    std::vector<std::pair<std::vector<long>, std::vector<int>>> seen;  // runs launched once so far
    bool tuning = false;               // autotuner trials: launch directly, no capture
    long cell_updates = 0;
    // device checkpoint (shll_checkpoint)
    void* ck_hi[2] = {nullptr, nullptr};
    float* ck_lo[2] = {nullptr, nullptr};
    std::vector<int> ck_par;
    long ck_updates = 0;
    // 2D engine (mixed2d.cu)
    void* d2 = nullptr;
};

// ---- autotuner choices, process-wide, by size class ----
// A class is (order, limiter, lam a power of two, state format, floor(log2(cells))); its choice is
// the sweep length B, the sweeps per fold window and the owned cells per chunk (0: the largest).
struct TuneKey {
    int order, limiter, pow2, kahan, lg;
    bool operator<(const TuneKey& o) const {
        if (order != o.order) return order < o.order;
        if (limiter != o.limiter) return limiter < o.limiter;
        if (pow2 != o.pow2) return pow2 < o.pow2;
        if (kahan != o.kahan) return kahan < o.kahan;
        return lg < o.lg;
    }
};
struct TuneVal { int B, fold_sweeps, owned; };
static std::mutex g_tune_mu;
static std::map<TuneKey, TuneVal> g_tune;

static TuneKey tune_key(const TubeP& tp, bool kahan) {
    int lg = 0;
    while ((2 << lg) <= tp.n) lg++;
    return {tp.order, tp.order == 2 ? tp.limiter : 0, tp.lam_pow2, kahan ? 1 : 0, lg};
}
static void apply_tuning(TubeP& tp, bool kahan) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(tune_key(tp, kahan));
    if (it == g_tune.end()) return;
    tp.B = it->second.B;
    tp.fold_sweeps = it->second.fold_sweeps;
    tp.owned = it->second.owned;
}

// owned cells per chunk: the window (MW) minus the halo on both sides, or the tube's tuned
// smaller size
static int chunk_owned(const TubeP& tp) {
    const int S = MW - 2 * tp.order * tp.B;
    return tp.owned > 0 && tp.owned < S ? tp.owned : S;
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
        const int S = chunk_owned(tp);
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

// fold windows of several sweeps need every halo cell to come from the adjacent chunk
static void fix_fold_sweeps(MixedState* m) {
    std::vector<int> min_owned(m->nitems, 1 << 30);
    for (const Chunk& c : m->chunks) min_owned[c.tube] = std::min(min_owned[c.tube], c.b - c.a);
    for (int t = 0; t < m->nitems; t++)
        if (min_owned[t] < m->tubes[t].order * m->tubes[t].B) m->tubes[t].fold_sweeps = 1;
}

// pair-flux flags per chunk and sweep parity
static cudaError_t alloc_mode_flags(MixedState* m) {
    for (int b = 0; b < 2; b++) { cudaFree(m->mode[b]); m->mode[b] = nullptr; }
    m->has_first = false;
    for (const TubeP& tp : m->tubes) m->has_first = m->has_first || tp.order == 1;
    for (int b = 0; b < 2; b++) {
        cudaError_t e = cudaMalloc(&m->mode[b], sizeof(int) * m->chunks.size());
        if (e == cudaSuccess) e = cudaMemset(m->mode[b], 0, sizeof(int) * m->chunks.size());
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
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
    bool windows = false;
    for (const TubeP& tp : m->tubes) windows = windows || tp.fold_sweeps > 1;
    if (windows) {
        for (int b = 0; b < 2; b++)
            if (cudaMalloc(&m->dh[b], cells * sizeof(float)) != cudaSuccess ||
                cudaMalloc(&m->dl[b], cells * sizeof(float)) != cudaSuccess) {
                snprintf(err, len, "cudaMalloc of deviation planes failed");
                return SHLL_ERR_NOMEM;
            }
        if (cudaMalloc(&m->frames, sizeof(Frame1) * m->chunks.size()) != cudaSuccess) {
            snprintf(err, len, "cudaMalloc of the frame table failed");
            return SHLL_ERR_NOMEM;
        }
    }
    if (cudaMalloc(&m->d_item_flags, sizeof(int) * m->nitems) != cudaSuccess ||
        cudaMemset(m->d_item_flags, 0, sizeof(int) * m->nitems) != cudaSuccess) {
        snprintf(err, len, "cudaMalloc of item flags failed");
        return SHLL_ERR_NOMEM;
    }
    if (alloc_mode_flags(m) != cudaSuccess) {
        snprintf(err, len, "cudaMalloc of the pair-flux flags failed");
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

// device descriptor of one tube (cells from `base` in the planes)
static TubeP tube_params(const shll_params& p, long base) {
    TubeP tp;
    memset(&tp, 0, sizeof(tp));
    tp.base = base;
    tp.n = p.nx;
    tp.order = p.order;
    tp.limiter = p.limiter;
    tp.gamma = p.gamma;
    tp.R = p.R;
    double lamy;
    item_consts(p, &tp.CV, &tp.lam, &lamy);
    tp.RoCV = tp.R / tp.CV;
    tp.gRf = (float)(tp.gamma * tp.R);
    tp.Rf = (float)tp.R;
    tp.cvinvf = (float)(1.0 / tp.CV);
    tp.alpha = (float)p.mc_alpha;
    const double pairs[2] = {tp.gamma * tp.RoCV, tp.RoCV};
    float* outs[2] = {tp.gg1p, tp.gm1p};
    for (int q = 0; q < 2; q++) {
        outs[q][0] = (float)pairs[q];
        outs[q][1] = (float)(pairs[q] - (double)outs[q][0]);
    }
    int ex;
    tp.lam_pow2 = std::frexp(tp.lam, &ex) == 0.5 && ex > -100 && ex < 100;
    tp.steps = 0;
    tp.par = 0;
    tp.fold_sweeps = 1;
    return tp;
}

MixedState* mixed2d_attach(MixedState* m, char* err, size_t len);  // mixed2d.cu
void mixed2d_detach(MixedState* m);
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
    const int fold = items[0].fold_steps > 0 ? items[0].fold_steps
                                             : (items[0].dim == 2 ? kDefaultFold2D : kDefaultFold1D);
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
    // sweep length B (temporal blocking depth) and sweeps per fold window: the FP64 state is read
    // and written once per fold window of (fold / B) * B steps
    m->B = std::min(fold, kSweepSteps);
    const int fold_sweeps = std::max(1, fold / m->B);
    long off = 0;
    for (int t = 0; t < count; t++) {
        const shll_params& p = items[t];
        TubeP tp = tube_params(p, off);
        tp.B = m->B;
        tp.fold_sweeps = fold_sweeps;
        if (items[t].fold_steps <= 0) apply_tuning(tp, m->kahan);   // a tuned choice of this size class
        m->tubes.push_back(tp);
        off += p.nx;
    }
    m->plane = off;
    m->par.assign(count, 0);
    build_chunks(m);
    fix_fold_sweeps(m);
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
        cudaFree(m->dh[b]); cudaFree(m->dl[b]);
    }
    cudaFree(m->frames);
    cudaFree(m->mode[0]);
    cudaFree(m->mode[1]);
    cudaFree(m->prog);
    cudaFree(m->stage);
    cudaFree(m->d_bad);
    cudaFree(m->d_bad_items);
    for (auto& g : m->graphs) cudaGraphExecDestroy(g.exec);
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

// ---- conversions between primitive planes and the stored state, on the device ----
// The FP64 arithmetic of Compute_U_from_P (base_shll.c:76-80, base_shll_2d.c:126-136) and of
// Compute_P_from_U (base_shll.c:171-176, base_shll_2d.c:312-318), in the operation order of a
// host FP64 evaluation of the same expressions (this unit is compiled without fused multiply-add
// and uses IEEE division, so the results are the host's bit for bit).

// the lowest cell index whose density or temperature is not positive, stored as n - 1 - i by an
// atomic maximum (-1: none)
__global__ void k_check_prim(const double* __restrict__ prim, long n, int nv, int* worst) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const double r = prim[i], T = prim[(long)(nv - 1) * n + i];
        if (!(r > 0.0) || !(T > 0.0)) {
            atomicMax(worst, (int)(n - 1 - i));
            break;  // (a thread's later cells have higher indices)
        }
    }
}

template <bool KAHAN>
__global__ void k_u_from_prim(const double* __restrict__ prim, MixedPlanes s) {
    const long n = s.n;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double U[4];
        const double p0 = prim[i], p1 = prim[n + i], p2 = prim[2 * n + i];
        U[0] = p0;
        U[1] = p0 * p1;
        if (s.nv == 3) {
            U[2] = p0 * (p2 * s.CV + 0.5 * p1 * p1);
        } else {
            const double p3 = prim[3 * n + i];
            U[2] = p0 * p2;
            U[3] = p0 * (p3 * s.CV + 0.5 * (p1 * p1 + p2 * p2));
        }
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (k >= s.nv) break;
            const long idx = k * s.plane + s.base + i;
            if (KAHAN) {
                const float h = __double2float_rn(U[k]);
                static_cast<float*>(s.hi)[idx] = h;
                s.lo[idx] = __double2float_rn(U[k] - (double)h);
            } else {
                static_cast<double*>(s.hi)[idx] = U[k];
            }
        }
    }
}

template <bool KAHAN>
__global__ void k_prim_from_u(MixedPlanes s, double* __restrict__ out) {
    const long n = s.n;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        double U[4];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (k >= s.nv) break;
            const long idx = k * s.plane + s.base + i;
            U[k] = KAHAN ? (double)static_cast<const float*>(s.hi)[idx] + (double)s.lo[idx]
                         : static_cast<const double*>(s.hi)[idx];
        }
        const double u0 = U[0], p1 = U[1] / u0;
        out[i] = u0;
        out[n + i] = p1;
        if (s.nv == 3) {
            out[2 * n + i] = ((U[2] / u0) - 0.5 * p1 * p1) / s.CV;
        } else {
            const double p2 = U[2] / u0;
            out[2 * n + i] = p2;
            out[3 * n + i] = ((U[3] / u0) - 0.5 * (p1 * p1 + p2 * p2)) / s.CV;
        }
    }
}

static int conv_grid(long n) { return (int)std::max(1L, std::min((n + 255) / 256, (long)device_sms() * 16)); }

// device staging area for nv planes of one item
static int ensure_stage(MixedState* m, size_t words, char* err, size_t len) {
    if (m->stage_words >= words && m->d_bad) return SHLL_OK;
    cudaFree(m->stage);
    m->stage = nullptr;
    m->stage_words = 0;
    if (cudaMalloc(&m->stage, words * sizeof(double)) != cudaSuccess ||
        (!m->d_bad && cudaMalloc(&m->d_bad, sizeof(int)) != cudaSuccess)) {
        cudaGetLastError();
        snprintf(err, len, "cudaMalloc of %zu staging values failed", words);
        return SHLL_ERR_NOMEM;
    }
    m->stage_words = words;
    return SHLL_OK;
}

// host primitive planes -> stored state of one item (check: refuse non-positive density or
// temperature first, leaving the state as it was)
static int upload_prim(MixedState* m, const MixedPlanes& s, const double* const* planes, bool check, char* err,
                       size_t len) {
    const size_t n = (size_t)s.n;
    int rc = ensure_stage(m, (size_t)s.nv * n, err, len);
    if (rc != SHLL_OK) return rc;
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < s.nv && e == cudaSuccess; k++)
        e = cudaMemcpyAsync(m->stage + k * n, planes[k], n * sizeof(double), cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess && check) {
        int worst = -1;
        e = cudaMemsetAsync(m->d_bad, 0xff, sizeof(int), m->stream);
        if (e == cudaSuccess) k_check_prim<<<conv_grid(s.n), 256, 0, m->stream>>>(m->stage, s.n, s.nv, m->d_bad);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&worst, m->d_bad, sizeof(int), cudaMemcpyDeviceToHost, m->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
        if (e == cudaSuccess && worst >= 0) {
            snprintf(err, len, "cell %ld: density and temperature must be positive", s.n - 1 - worst);
            return SHLL_ERR_ARG;
        }
    }
    if (e == cudaSuccess) {
        if (s.kahan) k_u_from_prim<true><<<conv_grid(s.n), 256, 0, m->stream>>>(m->stage, s);
        else k_u_from_prim<false><<<conv_grid(s.n), 256, 0, m->stream>>>(m->stage, s);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) { snprintf(err, len, "state upload failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    return SHLL_OK;
}

// stored state of one item -> host primitive planes (null pointers are skipped)
static int download_prim(MixedState* m, const MixedPlanes& s, double* const* out, char* err, size_t len) {
    const size_t n = (size_t)s.n;
    int rc = ensure_stage(m, (size_t)s.nv * n, err, len);
    if (rc != SHLL_OK) return rc;
    if (s.kahan) k_prim_from_u<true><<<conv_grid(s.n), 256, 0, m->stream>>>(s, m->stage);
    else k_prim_from_u<false><<<conv_grid(s.n), 256, 0, m->stream>>>(s, m->stage);
    cudaError_t e = cudaGetLastError();
    for (int k = 0; k < s.nv && e == cudaSuccess; k++)
        if (out[k]) e = cudaMemcpyAsync(out[k], m->stage + k * n, n * sizeof(double), cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e != cudaSuccess) { snprintf(err, len, "state download failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    return SHLL_OK;
}

// where item t's state lies (1D: buffer `buf`)
static MixedPlanes item_planes(MixedState* m, int t, int buf) {
    MixedPlanes s;
    if (m->dim == 2) {
        mixed2d_planes(m, t, &s);
        return s;
    }
    const TubeP& tp = m->tubes[t];
    s.hi = m->hi[buf];
    s.lo = m->lo[buf];
    s.base = tp.base;
    s.plane = m->plane;
    s.n = tp.n;
    s.nv = 3;
    s.kahan = m->kahan;
    s.CV = tp.CV;
    return s;
}

// one item's state from primitive planes (1D tubes start in buffer 0)
static int load_item(MixedState* m, int t, const double* const* planes, bool check, char* err, size_t len) {
    int rc = upload_prim(m, item_planes(m, t, 0), planes, check, err, len);
    if (rc == SHLL_OK && m->dim == 1) m->par[t] = 0;
    return rc;
}

static void plane_ptrs(const double* prim, long n, int nv, const double* out[4]) {
    for (int k = 0; k < 4; k++) out[k] = k < nv ? prim + k * n : nullptr;
}

int mixed_load(MixedState* m, const double* prim, char* err, size_t len) {
    cudaMemsetAsync(m->d_flag, 0, sizeof(int), m->stream);
    cudaMemsetAsync(m->d_item_flags, 0, sizeof(int) * m->nitems, m->stream);
    const MixedPlanes s = item_planes(m, 0, 0);
    const double* planes[4];
    plane_ptrs(prim, s.n, s.nv, planes);
    int rc = load_item(m, 0, planes, false, err, len);
    if (rc == SHLL_OK && cudaStreamSynchronize(m->stream) != cudaSuccess) {
        snprintf(err, len, "state upload failed");
        return SHLL_ERR_CUDA;
    }
    return rc;
}

int mixed_load_all(MixedState* m, char* err, size_t len) {
    cudaMemsetAsync(m->d_flag, 0, sizeof(int), m->stream);
    cudaMemsetAsync(m->d_item_flags, 0, sizeof(int) * m->nitems, m->stream);
    std::vector<double> prim;
    for (int t = 0; t < m->nitems; t++) {
        const shll_params& p = m->items[t];
        const int nv = p.dim == 2 ? 4 : 3;
        const long n = (long)p.nx * (p.dim == 2 ? p.ny : 1);
        prim.resize((size_t)nv * n);
        shll_ic_fill(&p, 64, prim.data());
        const double* planes[4];
        plane_ptrs(prim.data(), n, nv, planes);
        // (a pageable source is copied before the call returns, so the vector can be refilled)
        int rc = load_item(m, t, planes, false, err, len);
        if (rc != SHLL_OK) return rc;
    }
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) { snprintf(err, len, "state upload failed"); return SHLL_ERR_CUDA; }
    return SHLL_OK;
}

// every item at once: `prim` holds, item after item, each item's nv planes of n doubles
static std::vector<long> packed_offsets(MixedState* m) {
    std::vector<long> off(m->nitems + 1, 0);
    for (int t = 0; t < m->nitems; t++) {
        const MixedPlanes s = item_planes(m, t, 0);
        off[t + 1] = off[t] + (long)s.nv * s.n;
    }
    return off;
}

int mixed_set_all_primitives(MixedState* m, const double* prim, char* err, size_t len) {
    const std::vector<long> off = packed_offsets(m);
    int rc = ensure_stage(m, (size_t)off[m->nitems], err, len);
    if (rc != SHLL_OK) return rc;
    if (!m->d_bad_items && cudaMalloc(&m->d_bad_items, sizeof(int) * m->nitems) != cudaSuccess) {
        cudaGetLastError();
        snprintf(err, len, "cudaMalloc of the check flags failed");
        return SHLL_ERR_NOMEM;
    }
    cudaError_t e = cudaMemcpyAsync(m->stage, prim, sizeof(double) * off[m->nitems], cudaMemcpyHostToDevice, m->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(m->d_bad_items, 0xff, sizeof(int) * m->nitems, m->stream);
    for (int t = 0; t < m->nitems && e == cudaSuccess; t++) {
        const MixedPlanes s = item_planes(m, t, 0);
        k_check_prim<<<conv_grid(s.n), 256, 0, m->stream>>>(m->stage + off[t], s.n, s.nv, m->d_bad_items + t);
    }
    std::vector<int> worst(m->nitems, -1);
    if (e == cudaSuccess) e = cudaMemcpyAsync(worst.data(), m->d_bad_items, sizeof(int) * m->nitems, cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e != cudaSuccess) { snprintf(err, len, "state upload failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    for (int t = 0; t < m->nitems; t++)
        if (worst[t] >= 0) {
            snprintf(err, len, "item %d, cell %ld: density and temperature must be positive", t,
                     item_planes(m, t, 0).n - 1 - worst[t]);
            return SHLL_ERR_ARG;
        }
    for (int t = 0; t < m->nitems; t++) {
        const MixedPlanes s = item_planes(m, t, 0);
        if (s.kahan) k_u_from_prim<true><<<conv_grid(s.n), 256, 0, m->stream>>>(m->stage + off[t], s);
        else k_u_from_prim<false><<<conv_grid(s.n), 256, 0, m->stream>>>(m->stage + off[t], s);
        if (m->dim == 1) m->par[t] = 0;
    }
    cudaMemsetAsync(m->d_flag, 0, sizeof(int), m->stream);
    cudaMemsetAsync(m->d_item_flags, 0, sizeof(int) * m->nitems, m->stream);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e != cudaSuccess) { snprintf(err, len, "state upload failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    return SHLL_OK;
}

int mixed_get_all_primitives(MixedState* m, double* prim, char* err, size_t len) {
    const std::vector<long> off = packed_offsets(m);
    int rc = ensure_stage(m, (size_t)off[m->nitems], err, len);
    if (rc != SHLL_OK) return rc;
    for (int t = 0; t < m->nitems; t++) {
        const MixedPlanes s = item_planes(m, t, m->dim == 1 ? m->par[t] : 0);
        if (s.kahan) k_prim_from_u<true><<<conv_grid(s.n), 256, 0, m->stream>>>(s, m->stage + off[t]);
        else k_prim_from_u<false><<<conv_grid(s.n), 256, 0, m->stream>>>(s, m->stage + off[t]);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(prim, m->stage, sizeof(double) * off[m->nitems], cudaMemcpyDeviceToHost, m->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
    if (e != cudaSuccess) { snprintf(err, len, "state download failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    return SHLL_OK;
}

int mixed_set_item_primitives(MixedState* m, int item, const double* const* planes, char* err, size_t len) {
    if (item < 0 || item >= m->nitems) { snprintf(err, len, "item %d out of range", item); return SHLL_ERR_ARG; }
    int rc = load_item(m, item, planes, true, err, len);
    if (rc != SHLL_OK) return rc;
    cudaMemsetAsync(m->d_flag, 0, sizeof(int), m->stream);
    cudaMemsetAsync(m->d_item_flags + item, 0, sizeof(int), m->stream);
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) { snprintf(err, len, "state upload failed"); return SHLL_ERR_CUDA; }
    return SHLL_OK;
}

static std::atomic<int> g_graph_replay{1};
extern "C" void shll_set_graph_replay(int on) { g_graph_replay = on ? 1 : 0; }
bool mixed_graph_replay_on(MixedState* m) { return g_graph_replay.load() != 0 && !m->tuning; }
void mixed_set_tuning(MixedState* m, bool on) { m->tuning = on; }
static std::atomic<int> g_resident{1};
extern "C" void shll_set_resident(int on) { g_resident = on ? 1 : 0; }
static std::atomic<int> g_stall{-1};
extern "C" void shll_debug_stall_chunk(int chunk) { g_stall = chunk; }
static std::atomic<int> g_pair_flux{1};
extern "C" void shll_set_pair_flux(int on) { g_pair_flux = on == 2 ? 2 : (on ? 1 : 0); }

// issues the launches of one run on m->stream: the sweeps of every variant group (or, resident,
// one launch for all sweeps of the run's single variant group), then the fix-up
// cluster > 0: the cluster form of a resident run, clusters of that many chunks (one tube each)
static cudaError_t issue_run(MixedState* m, const std::vector<Chunk>& order, long nsweeps, long* launches,
                             bool resident = false, int cluster = 0) {
    struct Group { int variant, first; std::vector<int> active; };
    std::vector<Group> groups;
    for (int c = 0; c < (int)order.size(); c++) {
        const TubeP& tp = m->tubes[order[c].tube];
        const int v = tube_variant(tp);
        if (groups.empty() || groups.back().variant != v) groups.push_back({v, c, std::vector<int>(nsweeps + 1, 0)});
        // active[k] = chunks of the group whose tube still has sweep k (suffix sum of a histogram)
        groups.back().active[(tp.steps + tp.B - 1) / tp.B]++;
    }
    for (Group& g : groups)
        for (long k = nsweeps - 1; k >= 0; k--) g.active[k] += g.active[k + 1];
    SweepArgs A;
    A.tubes = m->d_tubes;
    A.chunks = m->d_chunks;
    A.hi[0] = m->hi[0]; A.hi[1] = m->hi[1];
    A.lo[0] = m->lo[0]; A.lo[1] = m->lo[1];
    A.bsum[0] = m->bsum[0]; A.bsum[1] = m->bsum[1];
    A.dh[0] = m->dh[0]; A.dh[1] = m->dh[1];
    A.dl[0] = m->dl[0]; A.dl[1] = m->dl[1];
    A.frames = m->frames;
    A.plane = m->plane;
    A.flag = m->d_flag;
    A.item_flags = m->d_item_flags;
    A.stall_id = resident ? g_stall.load() : -1;
    A.sweep = 0;
    const int pf = g_pair_flux.load();
    const bool pairs = pf && m->mode[0] && (m->has_first || pf == 2);
    A.mode[0] = pairs ? m->mode[0] : nullptr;
    A.mode[1] = pairs ? m->mode[1] : nullptr;
    A.pair_m2 = pf == 2 ? -1.0f : kPairMach * kPairMach;
    long n = 0, extra = 0;
    if (pairs) {  // the flags of the state at the start of the run
        A.chunk0 = 0;
        if (m->kahan) k_mode1d<true><<<(unsigned)order.size(), 256, 0, m->stream>>>(A);
        else k_mode1d<false><<<(unsigned)order.size(), 256, 0, m->stream>>>(A);
        extra++;
    }
    if (cluster > 0) {
        A.chunk0 = 0;
        const cudaError_t e = launch_cluster(groups[0].variant, m->kahan, (int)order.size(), cluster, m->stream, A, false);
        if (e != cudaSuccess) return e;
        n = 1;
        nsweeps = 0;
    } else if (resident) {
        A.chunk0 = 0;
        cudaError_t e = cudaMemsetAsync(m->prog, 0, sizeof(unsigned) * kProgStride * order.size(), m->stream);
        if (e == cudaSuccess)
            e = launch_resident(groups[0].variant, m->kahan, (int)order.size(), m->stream, A, m->prog, false,
                                pairs && pf == 2);
        if (e != cudaSuccess) return e;
        n = 1;
        nsweeps = 0;
    }
    for (long k = 0; k < nsweeps; k++) {
        A.sweep = (int)k;
        for (const Group& g : groups) {
            const int cnt = g.active[k + 1];
            if (cnt == 0) continue;
            A.chunk0 = g.first;
            // the FP32 form (not needed when every chunk takes the pair flux), then the same
            // chunks' pair-flux form (first order, or every order when asked for everywhere)
            cudaError_t e = cudaSuccess;
            if (!(pairs && pf == 2)) {
                e = launch_sweep(g.variant, m->kahan, cnt, m->stream, A, n > 0);
                if (e != cudaSuccess) return e;
                n++;
            }
            if (pairs && (g.variant <= 1 || pf == 2)) {
                e = launch_sweep_ff(g.variant, m->kahan, cnt, m->stream, A, n > 0);
                if (e != cudaSuccess) return e;
                n++;
            }
        }
    }
    A.chunk0 = 0;
    const int nch = (int)order.size();
    if (m->kahan) k_fixup1d<true><<<(nch + 127) / 128, 128, 0, m->stream>>>(A, nch);
    else k_fixup1d<false><<<(nch + 127) / 128, 128, 0, m->stream>>>(A, nch);
    *launches = n + extra + 1;
    return cudaGetLastError();
}


// A run is resident (k_tube1d) when its chunks fit on the GPU at once with one block per SM (the
// single-wave, latency-bound case: a tube of up to about 68000 cells), share one scheme variant,
// and each chunk owns at least the halo width, so that every halo cell comes from an adjacent
// chunk.  Larger runs keep one launch per sweep, which fills the SMs with several blocks each.
static std::atomic<int> g_cluster{0};
extern "C" void shll_set_cluster_runs(int on) { g_cluster = on ? 1 : 0; }

// The cluster form applies when asked for (shll_set_cluster_runs) to runs whose tubes share one scheme
// variant and one chunk count k (2 <= k <= 16, consecutive in `order`), every chunk owning at least
// the halo width, and not in the pair flux everywhere; returns k, or 0.
static int cluster_run(MixedState* m, const std::vector<Chunk>& order) {
    if (!g_cluster.load() || order.empty() || g_pair_flux.load() == 2) return 0;
    const int v = tube_variant(m->tubes[order[0].tube]);
    int k = 0;
    for (size_t c = 0; c < order.size();) {
        const int t = order[c].tube;
        size_t e = c;
        while (e < order.size() && order[e].tube == t) e++;
        const int kt = (int)(e - c);
        if (k == 0) k = kt;
        if (kt != k || kt < 2 || kt > 16) return 0;
        for (size_t q = c; q < e; q++) {
            const TubeP& tp = m->tubes[order[q].tube];
            if (tube_variant(tp) != v || order[q].b - order[q].a < tp.order * tp.B || order[q].id != order[c].id + (int)(q - c))
                return 0;
        }
        c = e;
    }
    SweepArgs none{};
    if (launch_cluster(v, m->kahan, (int)order.size(), k, m->stream, none, true) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return k;
}

static bool resident_run(MixedState* m, const std::vector<Chunk>& order) {
    if (!g_resident.load() || order.empty() || (long)order.size() > device_sms()) return false;
    const int v = tube_variant(m->tubes[order[0].tube]);
    for (const Chunk& c : order) {
        const TubeP& tp = m->tubes[c.tube];
        if (tube_variant(tp) != v || c.b - c.a < tp.order * tp.B) return false;
    }
    if (m->prog_n < order.size()) {
        cudaFree(m->prog);
        m->prog = nullptr;
        m->prog_n = 0;
        if (cudaMalloc(&m->prog, sizeof(unsigned) * kProgStride * order.size()) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        m->prog_n = order.size();
    }
    SweepArgs none{};
    if (launch_resident(v, m->kahan, (int)order.size(), m->stream, none, m->prog, true, g_pair_flux.load() == 2) !=
        cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return true;
}

// advances every tube by `steps[t]` steps (one launch per sweep of B steps).  A run whose step
// counts and buffer parities occur for the second time is captured into a CUDA graph, which later
// identical runs replay (the descriptors are uploaded before either); a run that occurs once is
// launched directly and pays no capture.
static int run_tubes(MixedState* m, const std::vector<long>& steps, char* err, size_t len) {
    long maxsteps = 0;
    for (int t = 0; t < m->nitems; t++) {
        m->tubes[t].steps = (int)steps[t];
        m->tubes[t].par = m->par[t];
        maxsteps = std::max(maxsteps, steps[t]);
    }
    if (maxsteps == 0) return SHLL_OK;
    // chunks grouped by scheme variant and, inside a group, ordered by their tube's sweep count,
    // so that the launch of sweep k for a group covers a prefix of the group
    std::vector<Chunk> order = m->chunks;
    auto sweeps_of = [&](const TubeP& tp) { return (tp.steps + tp.B - 1) / tp.B; };
    std::stable_sort(order.begin(), order.end(), [&](const Chunk& x, const Chunk& y) {
        const int vx = tube_variant(m->tubes[x.tube]), vy = tube_variant(m->tubes[y.tube]);
        if (vx != vy) return vx < vy;
        return sweeps_of(m->tubes[x.tube]) > sweeps_of(m->tubes[y.tube]);
    });
    if (cudaMemcpyAsync(m->d_tubes, m->tubes.data(), sizeof(TubeP) * m->nitems, cudaMemcpyHostToDevice, m->stream) != cudaSuccess ||
        cudaMemcpyAsync(m->d_chunks, order.data(), sizeof(Chunk) * order.size(), cudaMemcpyHostToDevice, m->stream) != cudaSuccess) {
        snprintf(err, len, "descriptor upload failed");
        return SHLL_ERR_CUDA;
    }
    long nsweeps = 0;
    for (const TubeP& tp : m->tubes) nsweeps = std::max(nsweeps, (long)sweeps_of(tp));
    long launches = 0;
    cudaError_t e = allow_solo_padding();
    if (e != cudaSuccess) { snprintf(err, len, "kernel attribute: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    MixedState::GraphEntry* hit = nullptr;
    const int cluster = cluster_run(m, order);
    const bool resident = !cluster && resident_run(m, order);
    // (a resident or cluster run is one launch: nothing to gain from a graph)
    const bool replay = g_graph_replay.load() != 0 && !m->tuning && !resident && !cluster;
    if (replay)
        for (auto& g : m->graphs)
            if (g.steps == steps && g.par == m->par) hit = &g;
    if (hit) {
        e = cudaGraphLaunch(hit->exec, m->stream);
        launches = hit->launches;
    } else {
        bool done = false;
        bool repeat = false;
        for (auto& k : m->seen) repeat = repeat || (k.first == steps && k.second == m->par);
        if (replay && !repeat) {
            if (m->seen.size() >= 8) m->seen.erase(m->seen.begin());
            m->seen.push_back({steps, m->par});
        }
        if (replay && repeat && m->stream != nullptr) {  // (the legacy default stream cannot be captured)
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            if (cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                const cudaError_t ei = issue_run(m, order, nsweeps, &launches);
                const cudaError_t ec = cudaStreamEndCapture(m->stream, &graph);
                if (ei == cudaSuccess && ec == cudaSuccess && graph &&
                    cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess) {
                    if (m->graphs.size() >= 4) {
                        cudaGraphExecDestroy(m->graphs.front().exec);
                        m->graphs.erase(m->graphs.begin());
                    }
                    m->graphs.push_back({steps, m->par, exec, launches});
                    e = cudaGraphLaunch(exec, m->stream);
                    done = true;
                }
                if (graph) cudaGraphDestroy(graph);
            }
            if (!done) cudaGetLastError();  // capture not possible here: launch directly
        }
        if (!done) e = issue_run(m, order, nsweeps, &launches, resident, cluster);
    }
    if (e != cudaSuccess) { snprintf(err, len, "sweep launch failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    shll_count_launches(launches);
    for (int t = 0; t < m->nitems; t++) {
        long sw = (steps[t] + m->tubes[t].B - 1) / m->tubes[t].B;
        m->par[t] = (int)((m->par[t] + sw) & 1);
        m->cell_updates += steps[t] * (long)m->tubes[t].n;
    }
    return SHLL_OK;
}

// re-chunks every tube after a change of sweep lengths or chunk sizes (descriptors, boundary
// sums, frame table; captured launch sequences are dropped)
static int rebuild_chunks(MixedState* m, char* err, size_t len) {
    for (TubeP& tp : m->tubes) tp.fold_sweeps = std::max(tp.fold_sweeps, 1);
    build_chunks(m);
    fix_fold_sweeps(m);
    for (auto& g : m->graphs) cudaGraphExecDestroy(g.exec);
    m->graphs.clear();
    m->seen.clear();
    const size_t nch = m->chunks.size();
    cudaFree(m->d_chunks); m->d_chunks = nullptr;
    cudaFree(m->frames); m->frames = nullptr;
    for (int b = 0; b < 2; b++) { cudaFree(m->bsum[b]); m->bsum[b] = nullptr; }
    bool ok = cudaMalloc(&m->d_chunks, sizeof(Chunk) * nch) == cudaSuccess &&
              cudaMalloc(&m->frames, sizeof(Frame1) * nch) == cudaSuccess &&
              cudaMalloc(&m->bsum[0], sizeof(BSum) * nch) == cudaSuccess &&
              cudaMalloc(&m->bsum[1], sizeof(BSum) * nch) == cudaSuccess;
    bool windows = false;
    for (const TubeP& tp : m->tubes) windows = windows || tp.fold_sweeps > 1;
    const size_t cells = (size_t)m->plane * 3;
    for (int b = 0; ok && windows && b < 2; b++)
        if (!m->dh[b])
            ok = cudaMalloc(&m->dh[b], cells * sizeof(float)) == cudaSuccess &&
                 cudaMalloc(&m->dl[b], cells * sizeof(float)) == cudaSuccess;
    ok = ok && alloc_mode_flags(m) == cudaSuccess;
    if (!ok) { snprintf(err, len, "re-chunking allocation failed"); return SHLL_ERR_NOMEM; }
    return SHLL_OK;
}

// Autotuner: picks, per size class, the sweep length B (the temporal-blocking depth, which sets a
// chunk's owned and halo cells) and the sweeps per FP64 fold window by timing short runs of this
// batch.  The state is checkpointed first and restored after every trial; the choices are kept
// in the process-wide table, so later batches and tubes of the same classes start with them.
int mixed2d_autotune(MixedState* m, int trial_steps, char* err, size_t len);   // mixed2d.cu
int mixed2d_checkpoint(MixedState* m, bool restore, char* err, size_t len);
int mixed2d_fold(MixedState* m);
int mixed2d_kstep(MixedState* m);

int mixed_autotune(MixedState* m, int trial_steps, char* err, size_t len) {
    if (m->dim == 2) {   // (the trials' cell updates and breakdown flags do not count)
        const long cu = m->cell_updates;
        const int rc = mixed2d_autotune(m, trial_steps, err, len);
        m->cell_updates = cu;
        if (m->d_flag) cudaMemsetAsync(m->d_flag, 0, sizeof(int), m->stream);
        if (m->d_item_flags) cudaMemsetAsync(m->d_item_flags, 0, sizeof(int) * m->nitems, m->stream);
        if (rc == SHLL_OK) m->ck_updates = cu;
        return rc;
    }
    long cells = 0;
    double work_total = 0;
    for (const TubeP& tp : m->tubes) { cells += tp.n; work_total += (double)tp.n * tp.n; }
    if (trial_steps <= 0) {  // about 4e8 cell-updates per trial, whole fold windows of up to 128 steps
        const long want = (long)(4e8 / (double)std::max(cells, 1L));
        trial_steps = (int)std::min(4096L, std::max(256L, (want + 255) / 256 * 256));
    }
    int rc = mixed_checkpoint(m, false, err, len);
    if (rc != SHLL_OK) return rc;
    m->tuning = true;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const std::vector<long> steps(m->nitems, trial_steps);
    // time of one trial: best of two runs from the checkpoint
    auto trial = [&](float* ms) -> int {
        int r = rebuild_chunks(m, err, len);
        float best = 1e30f;
        for (int rep = 0; r == SHLL_OK && rep < 2; rep++) {
            r = mixed_checkpoint(m, true, err, len);
            if (r != SHLL_OK) break;
            cudaEventRecord(e0, m->stream);
            r = run_tubes(m, steps, err, len);
            cudaEventRecord(e1, m->stream);
            if (cudaEventSynchronize(e1) != cudaSuccess) { snprintf(err, len, "trial failed"); r = SHLL_ERR_CUDA; }
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            best = std::min(best, t);
        }
        *ms = best;
        return r;
    };
    // owned cells per chunk: the largest window (0) or half of it (smaller chunks, more blocks per
    // SM: they hide each other's barriers and per-sweep latency at the cost of more halo work)
    struct Cand { int B, F, half; };
    std::vector<Cand> cands;
    for (int B : {8, 16, 32})
        for (int F : {1, 2, 4, 8})
            for (int half : {0, 1})
                if (B * F <= std::max(trial_steps, 128) && B <= MW / 16) cands.push_back({B, F, half});
    std::map<TuneKey, std::vector<int>> classes;
    for (int t = 0; t < m->nitems; t++) classes[tune_key(m->tubes[t], m->kahan)].push_back(t);
    // per class, the longest sweep whose chunks (window MW minus the halos) still number at most one
    // per SM for the class's largest tube: such a tube runs resident with every SM busy, and a longer
    // sweep spreads the per-sweep cost (records, neighbour wait, halo loads) over more steps (65536
    // cells, second order: 20 steps, 152 chunks of 431 cells)
    for (auto& kv : classes) {
        int nmax = 0, order = 1;
        for (int t : kv.second) { nmax = std::max(nmax, m->tubes[t].n); order = m->tubes[t].order; }
        const int per = (nmax + device_sms() - 1) / device_sms();
        const int Bfit = (MW - per) / (2 * order);
        if (Bfit > 8 && Bfit < MW / 16 && Bfit != 16)
            for (int F : {1, 2, 4, 8})
                if (Bfit * F <= std::max(trial_steps, 128)) {
                    bool dup = false;
                    for (const Cand& c : cands) dup = dup || (c.B == Bfit && c.F == F && c.half == 0);
                    if (!dup) cands.push_back({Bfit, F, 0});
                }
    }
    auto set_class = [&](const std::vector<int>& ts, Cand c) {
        for (int t : ts) {
            TubeP& tp = m->tubes[t];
            tp.B = c.B;
            tp.fold_sweeps = c.F;
            tp.owned = c.half ? std::max(2 * tp.order * c.B, (MW - 2 * tp.order * c.B) / 2) : 0;
        }
    };
    // 1) one choice for every class
    Cand best_all = {m->B, 1, 0};
    float best_ms = 1e30f;
    for (const Cand& c : cands) {
        for (auto& kv : classes) set_class(kv.second, c);
        float ms = 0;
        rc = trial(&ms);
        if (rc != SHLL_OK) break;
        if (ms < best_ms) { best_ms = ms; best_all = c; }
    }
    std::map<TuneKey, Cand> choice;
    for (auto& kv : classes) { set_class(kv.second, best_all); choice[kv.first] = best_all; }
    // 2) the classes that hold at least a tenth of the work, one at a time
    for (auto& kv : classes) {
        if (rc != SHLL_OK) break;
        double w = 0;
        for (int t : kv.second) w += (double)m->tubes[t].n * m->tubes[t].n;
        if (w < 0.1 * work_total || classes.size() == 1) continue;
        for (const Cand& c : cands) {
            if (c.B == choice[kv.first].B && c.F == choice[kv.first].F && c.half == choice[kv.first].half) continue;
            set_class(kv.second, c);
            float ms = 0;
            rc = trial(&ms);
            if (rc != SHLL_OK) break;
            if (ms < 0.99f * best_ms) { best_ms = ms; choice[kv.first] = c; }
        }
        set_class(kv.second, choice[kv.first]);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    m->tuning = false;
    if (rc == SHLL_OK) rc = rebuild_chunks(m, err, len);
    if (rc == SHLL_OK) rc = mixed_checkpoint(m, true, err, len);
    if (rc != SHLL_OK) return rc;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto& kv : choice) {
        const TubeP& tp = m->tubes[classes[kv.first][0]];
        g_tune[kv.first] = {kv.second.B, kv.second.F, tp.owned};
    }
    return SHLL_OK;
}

// sweep length and fold interval (steps) and owned cells per chunk chosen for a tube
int mixed_tuning(MixedState* m, int item, int* sweep_steps, int* fold_steps, int* chunk_cells) {
    if (item < 0 || item >= m->nitems) return SHLL_ERR_ARG;
    if (m->dim == 2) {   // steps per launch, one fold window for the batch, 16 x 32 tiles
        if (sweep_steps) *sweep_steps = mixed2d_kstep(m);
        if (fold_steps) *fold_steps = mixed2d_fold(m);
        if (chunk_cells) *chunk_cells = 16 * 32;
        return SHLL_OK;
    }
    const TubeP& tp = m->tubes[item];
    if (sweep_steps) *sweep_steps = tp.B;
    if (fold_steps) *fold_steps = tp.B * tp.fold_sweeps;
    if (chunk_cells) *chunk_cells = chunk_owned(tp);
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
    const MixedPlanes s = item_planes(m, item, m->dim == 1 ? m->par[item] : 0);
    double* const out3[3] = {rho, u, T};
    double* const out4[4] = {rho, u, v, T};
    return download_prim(m, s, s.nv == 3 ? out3 : out4, err, len);
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
    if (m->dim == 2) {
        int rc = mixed2d_checkpoint(m, restore, err, len);
        if (rc == SHLL_OK && restore) {
            m->cell_updates = m->ck_updates;
            if (m->d_flag) cudaMemsetAsync(m->d_flag, 0, sizeof(int), m->stream);
            if (m->d_item_flags) cudaMemsetAsync(m->d_item_flags, 0, sizeof(int) * m->nitems, m->stream);
        } else if (rc == SHLL_OK) {
            m->ck_updates = m->cell_updates;
        }
        return rc;
    }
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
    if (restore) {
        m->par = m->ck_par;
        m->cell_updates = m->ck_updates;
        // breakdown flags raised after the checkpoint no longer apply
        if (m->d_flag) cudaMemsetAsync(m->d_flag, 0, sizeof(int), m->stream);
        if (m->d_item_flags) cudaMemsetAsync(m->d_item_flags, 0, sizeof(int) * m->nitems, m->stream);
    } else {
        m->ck_par = m->par;
        m->ck_updates = m->cell_updates;
    }
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
constexpr size_t kStaticFlagOff = kStaticTubeOff + (sizeof(TubeP) + 255) / 256 * 256;
static_assert(kStaticFlagOff >= kStaticTubeOff + sizeof(TubeP), "the tube descriptor overlaps the error flag");
constexpr size_t kStaticModeOff = kStaticFlagOff + 256;                               // 2 x int[256]
constexpr size_t kStaticScratchBytes = 2u << 20;
static_assert(kStaticModeOff + 2 * kStaticMaxChunks * sizeof(int) <= kStaticScratchBytes,
              "static scratch layout exceeds its array");
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
    {   // the same parameter checks as shll_create, whatever nsteps is
        char msg[256];
        if (shll_validate_params(p, msg, sizeof(msg)) != SHLL_OK) {
            fprintf(stderr, "shll_tube_run_static: %s\n", msg);
            return SHLL_ERR_ARG;
        }
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
    const int fold = p->fold_steps > 0 ? p->fold_steps : kSweepSteps;
    const int B = std::min(fold, MW / 16);
    TubeP tp = tube_params(*p, 0);
    tp.B = B;
    tp.fold_sweeps = 1;
    tp.steps = (int)nsteps;
    tp.par = 0;
    Chunk chunks[kStaticMaxChunks];
    const int n = tp.n;
    const int S = chunk_owned(tp);
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
    A.dh[0] = A.dh[1] = A.dl[0] = A.dl[1] = nullptr;  // one sweep per fold window: no pairs, no frame table
    A.frames = nullptr;
    A.bsum[0] = reinterpret_cast<BSum*>(sc + kStaticBSumOff);
    A.bsum[1] = A.bsum[0] + kStaticMaxChunks;
    A.plane = n;
    A.flag = d_flag;
    A.item_flags = nullptr;
    A.stall_id = -1;
    A.chunk0 = 0;
    // first order: the pair-flux flags, as in the context API (two ints per chunk in the array;
    // the start-of-run kernel writes them before the first sweep reads them)
    const int pf = g_pair_flux.load();
    const bool pairs = pf && (tp.order == 1 || pf == 2);
    A.mode[0] = pairs ? reinterpret_cast<int*>(sc + kStaticModeOff) : nullptr;
    A.mode[1] = pairs ? A.mode[0] + kStaticMaxChunks : nullptr;
    A.pair_m2 = pf == 2 ? -1.0f : kPairMach * kPairMach;
    const long nsweeps = (nsteps + B - 1) / B;
    e = allow_solo_padding();
    if (e == cudaSuccess && pairs) {
        k_mode1d<false><<<k, 256, 0, s>>>(A);
        e = cudaGetLastError();
    }
    const bool fp32 = !(pairs && pf == 2);   // (every chunk takes the pair flux: no FP32 launches)
    shll_count_launches(((fp32 ? 1 : 0) + (pairs ? 1 : 0)) * nsweeps + (pairs ? 1 : 0) + 1);
    for (long w = 0; w < nsweeps && e == cudaSuccess; w++) {
        A.sweep = (int)w;
        if (fp32) e = launch_sweep(tube_variant(tp), false, k, s, A, w > 0);
        if (e == cudaSuccess && pairs) e = launch_sweep_ff(tube_variant(tp), false, k, s, A, fp32 || w > 0);
    }
    if (e != cudaSuccess) {
        fprintf(stderr, "shll_tube_run_static: sweep launch failed: %s\n", cudaGetErrorString(e));
        return SHLL_ERR_CUDA;
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

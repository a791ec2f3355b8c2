// Device helpers of the mixed-precision engine: FP32-pair (compensated) arithmetic and the
// split fluxes of a cell evaluated in FP32 as deviations from an anchor state.
//
// Split fluxes (base-c/base_shll.c:134-158):  M = u/a, Z1 = (M+1)/2, Z2 = a(1-M^2)/2,
// Z3 = (M-1)/2 = Z1 - 1, P = rho R T, F = (m, m u + P, u (E + P)),
// fp = F Z1 + U Z2, fm = -F Z3 - U Z2.  Every quantity q is written as q* + dq with q* the
// anchor value; the deviations obey exact identities, e.g.
//   du = (dm - u* drho)/rho,  de = (dE - e* drho)/rho,  dT = (de - (u + u*) du / 2)/CV,
//   da = gamma R dT/(a + a*),  dM = (du - M* da)/a,  dZ2 = (da (1-M^2) - a* (M + M*) dM)/2,
//   dP = (gamma-1)(dE - (dm u + m* du)/2),  dfp = dF Z1 + F* dZ1 + dU Z2 + U* dZ2,
//   dfm = dF - dfp,
// in which the anchor values only multiply deviations.  Rounding errors are therefore relative
// to |U - U*|; reciprocals and square roots may use the fast approximations.
#pragma once
#include <cuda_runtime.h>

struct AnchorCoef {
    float rho, u, v, e, T, a, M, P, Z1, Z2, gR, R, cvinv;
    float F[4], Uf[4];
};

// h + l += v (TwoSum; the rounding error goes to l)
__device__ __forceinline__ void two_sum_acc(float& h, float& l, float v) {
    float s = __fadd_rn(h, v);
    float bp = __fadd_rn(s, -h);
    float e = __fadd_rn(__fadd_rn(h, -__fadd_rn(s, -bp)), __fadd_rn(v, -bp));
    h = s;
    l = __fadd_rn(l, e);
}

__device__ __forceinline__ void split2(double d, float& h, float& l) {
    h = (float)d;
    l = (float)(d - (double)h);
}

// (oh, ol) = (ah + al) + (bh + bl), renormalised
__device__ __forceinline__ void ff_add(float ah, float al, float bh, float bl, float& oh, float& ol) {
    float s = __fadd_rn(ah, bh);
    float bp = __fadd_rn(s, -ah);
    float e = __fadd_rn(__fadd_rn(ah, -__fadd_rn(s, -bp)), __fadd_rn(bh, -bp));
    e = __fadd_rn(e, __fadd_rn(al, bl));
    oh = __fadd_rn(s, e);
    ol = __fadd_rn(e, -__fadd_rn(oh, -s));
}
__device__ __forceinline__ void ff_sub(float ah, float al, float bh, float bl, float& oh, float& ol) {
    ff_add(ah, al, -bh, -bl, oh, ol);
}

__device__ __forceinline__ float fast_rcp(float x) { return __fdividef(1.0f, x); }

// ---- packed FP32x2: two cells per thread, one f32x2 instruction per operation --------------
// (__fadd2_rn / __fmul2_rn / __ffma2_rn: the sm_100-family packed FP32 instructions, each lane
// rounded to nearest exactly like the scalar operation, so a packed lane and a scalar evaluation
// of the same formula give identical bits)
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
// a - b per lane: the packed subtract (sub.rn.f32x2), the same bits as a + (-b).  Written out
// because the compiler does not fold the negation of a packed operand into the packed add (the
// resident 1D sweep ran 1.5 % faster with this form on GB300)
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d)
        : "l"(*reinterpret_cast<const unsigned long long*>(&a)), "l"(*reinterpret_cast<const unsigned long long*>(&b)));
    return *reinterpret_cast<const float2*>(&d);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 rcp2(float2 a) { return make_float2(fast_rcp(a.x), fast_rcp(a.y)); }
__device__ __forceinline__ float2 rsqrt2(float2 a) { return make_float2(rsqrtf(a.x), rsqrtf(a.y)); }
// lane q of a float2 (q a compile-time constant after unrolling)
__device__ __forceinline__ float lane(float2 v, int q) { return q ? v.y : v.x; }
__device__ __forceinline__ void set_lane(float2& v, int q, float x) { if (q) v.y = x; else v.x = x; }

// h + l += v per lane (TwoSum)
__device__ __forceinline__ void two_sum_acc2(float2& h, float2& l, float2 v) {
    const float2 s = add2(h, v);
    const float2 bp = sub2(s, h);
    const float2 e = add2(sub2(h, sub2(s, bp)), sub2(v, bp));
    h = s;
    l = add2(l, e);
}
// h + l -= v per lane: the same bits as two_sum_acc2(h, l, -v) (negation commutes with rounding
// to nearest: (-v) - bp = -(v + bp))
__device__ __forceinline__ void two_diff_acc2(float2& h, float2& l, float2 v) {
    const float2 s = sub2(h, v);
    const float2 bp = sub2(s, h);
    const float2 e = sub2(sub2(h, sub2(s, bp)), add2(v, bp));
    h = s;
    l = add2(l, e);
}

// minmod(a, b): the smaller magnitude with the common sign when a and b have the same sign,
// else 0.  Three integer/min-max operations: t = min(|a|,|b|) carrying sign(a) xor sign(b)
// (PTX min.xorsign.abs), r = max(t, 0) (0 unless the signs agree), then sign(a) on r.
// Symmetric in a and b up to the sign of a zero result, so threads that evaluate the same slope
// get the same value.
__device__ __forceinline__ float minmod_s(float a, float b) {
    float t;
    asm("min.xorsign.abs.f32 %0, %1, %2;" : "=f"(t) : "f"(a), "f"(b));
    const float r = fmaxf(t, 0.f);
    return __uint_as_float(__float_as_uint(r) | (__float_as_uint(a) & 0x80000000u));
}
__device__ __forceinline__ float2 minmod2(float2 a, float2 b) {
    return make_float2(minmod_s(a.x, b.x), minmod_s(a.y, b.y));
}
// limited slope from the backward and forward differences a = f_j - f_{j-1}, b = f_{j+1} - f_j:
// minmod (LIM = 0) or the MC limiter minmod((a+b)/2, alpha minmod(a,b)) (LIM = 1,
// base-omp/2nd_order_base_shll.c:316-325)
template <int LIM>
__device__ __forceinline__ float slope_s(float a, float b, float alpha) {
    if (LIM == 1) return minmod_s(__fmul_rn(0.5f, __fadd_rn(a, b)), __fmul_rn(alpha, minmod_s(a, b)));
    return minmod_s(a, b);
}
template <int LIM>
__device__ __forceinline__ float2 slope2(float2 a, float2 b, float alpha) {
    if (LIM == 1) return minmod2(mul2(f2(0.5f), add2(a, b)), mul2(f2(alpha), minmod2(a, b)));
    return minmod2(a, b);
}

// anchor coefficients of a 1D frame, each duplicated into both lanes (negated where the
// formulas subtract them)
struct Coef2 {
    float2 rho, u, nu, ne, T, a, na, M, nM, Z1, Z2, P, gR, R, cvinv, gm1;
    float2 F[3], Uf[3];
};
__device__ __forceinline__ Coef2 coef2(const AnchorCoef& c) {
    Coef2 k;
    k.rho = f2(c.rho); k.u = f2(c.u); k.nu = f2(-c.u); k.ne = f2(-c.e); k.T = f2(c.T); k.a = f2(c.a); k.na = f2(-c.a);
    k.M = f2(c.M); k.nM = f2(-c.M); k.Z1 = f2(c.Z1); k.Z2 = f2(c.Z2); k.P = f2(c.P); k.gR = f2(c.gR);
    k.R = f2(c.R);
    k.cvinv = f2(c.cvinv);
    k.gm1 = f2(__fmul_rn(c.R, c.cvinv));   // R / CV = gamma - 1
    for (int i = 0; i < 3; i++) { k.F[i] = f2(c.F[i]); k.Uf[i] = f2(c.Uf[i]); }
    return k;
}

// 1D split-flux deviations of two cells at once (the conserved deviations d = (drho, dm, dE) of
// both cells as the lanes of FP32x2 registers)
__device__ __forceinline__ void dflux1x2(const Coef2& c, const float2 d[3], float2 dfp[3], float2 dfm[3]) {
    const float2 drho = d[0], dm = d[1], dE = d[2];
    const float2 rho = add2(c.rho, drho);
    const float2 r = rcp2(rho);
    const float2 du = mul2(fma2(c.nu, drho, dm), r);
    const float2 u = add2(c.u, du);
    const float2 de = mul2(fma2(c.ne, drho, dE), r);
    const float2 dT = mul2(fma2(f2(-0.5f), mul2(add2(u, c.u), du), de), c.cvinv);
    const float2 T = add2(c.T, dT);
    const float2 gRT = mul2(c.gR, T);
    const float2 ainv = rsqrt2(gRT);
    const float2 a = mul2(gRT, ainv);
    const float2 da = mul2(mul2(c.gR, dT), rcp2(add2(a, c.a)));
    const float2 dM = mul2(fma2(c.nM, da, du), ainv);
    const float2 M = add2(c.M, dM);
    const float2 dZ1 = mul2(f2(0.5f), dM);
    const float2 Z1 = add2(c.Z1, dZ1);
    // (negations folded into the operations: -M = (-M*) - dM and -(a* s dM) = ((-a*) s) dM, the
    // same bits as negating the results)
    const float2 omm = fma2(sub2(c.nM, dM), M, f2(1.0f));
    const float2 dZ2 = mul2(f2(0.5f), fma2(da, omm, mul2(mul2(c.na, add2(M, c.M)), dM)));
    const float2 Z2 = add2(c.Z2, dZ2);
    // P = (gamma-1)(E - m u / 2): dP = (gamma-1)(dE - (dm u + m* du) / 2).  At a contact (P and u
    // continuous) this cancels kinetic-energy-sized terms, where R (drho T + rho* dT) would cancel
    // internal-energy-sized ones
    const float2 dP = mul2(c.gm1, fma2(f2(-0.5f), fma2(dm, u, mul2(c.Uf[1], du)), dE));
    const float2 P = add2(c.P, dP);
    const float2 E = add2(c.Uf[2], dE);
    float2 dF[3];
    dF[0] = dm;
    dF[1] = add2(fma2(dm, u, mul2(c.Uf[1], du)), dP);
    dF[2] = fma2(du, add2(E, P), mul2(c.u, add2(dE, dP)));
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float2 a1 = fma2(dF[k], Z1, mul2(c.F[k], dZ1));
        const float2 a2 = fma2(d[k], Z2, mul2(c.Uf[k], dZ2));
        dfp[k] = add2(a1, a2);
        // fp + fm = F (Z1 - Z3 = 1).  Besides saving the minus-flux products, the difference keeps
        // dfp + dfm = dF to one rounding, which the separately rounded form -(dF Z3 + F* dZ1 + d Z2)
        // did not: on strong tubes with supersonic flow (where this split amplifies perturbations)
        // the FP32-flux error fell from about 1e-2 to 3e-6 against FP64
        dfm[k] = sub2(dF[k], dfp[k]);
    }
}

// ---- FP64 <-> FP32 conversions on the integer pipes --------------------------------------
// GB300 executes FP64 arithmetic and F2F conversions at 2 lanes per clock per SM, so the
// once-per-sweep conversions are done with bit operations instead (IEEE-754 layouts:
// float = s | e8 | m23, double = s | e11 | m52; exponent biases 127 and 1023).

// float -> double, exact for normal floats and zero; subnormal floats become signed zero,
// infinities and NaNs stay non-finite
__device__ __forceinline__ double f2d_bits(float f) {
    const unsigned b = __float_as_uint(f);
    const unsigned e = (b >> 23) & 0xffu;
    unsigned hi = (b & 0x80000000u) | (((b & 0x7fffffffu) >> 3) + ((1023u - 127u) << 20));
    unsigned lo = b << 29;
    if (e == 0u) { hi = b & 0x80000000u; lo = 0u; }
    if (e == 0xffu) hi |= 0x7ff00000u;
    return __hiloint2double((int)hi, (int)lo);
}

// double -> FP32 pair (h, l): h = x truncated to 24 significant bits, l = x - h (29 bits)
// rounded to nearest FP32, so |x - (h + l)| <= 2^-48 |x|.  |x| < 2^-126 gives (0, 0) and
// 2^-126 <= |x| < 2^-74 gives l = 0 (absolute error below 2^-97); |x| >= 2^128 and
// non-finite x give a NaN h.
__device__ __forceinline__ void d2ff_bits(double x, float& h, float& l) {
    const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
    const unsigned e = (hi >> 20) & 0x7ffu;
    const unsigned s = hi & 0x80000000u;
    // h: sign | (e - 896) << 23 | top 23 mantissa bits (20 from hi, 3 from lo)
    const unsigned hb = s | ((((hi & 0x7fffffffu) - (896u << 20)) << 3) & 0x7fffffffu) | (lo >> 29);
    // l: the low 29 mantissa bits as an integer r, times 2^(e - 1075); r is converted exactly in
    // two 23-bit halves through the 2^23 magic-number trick, the final fma rounds once
    const unsigned r = lo & 0x1fffffffu;
    const float rh = __fadd_rn(__uint_as_float(0x4b000000u | (r >> 6)), -8388608.0f);
    const float rl = __fadd_rn(__uint_as_float(0x4b000000u | (r & 63u)), -8388608.0f);
    const float rf = __fmaf_rn(rh, 64.0f, rl);
    const float scale = __uint_as_float((e - 948u) << 23);  // 2^(e - 1075), valid for e in [949, 1202]
    const float lf = __uint_as_float(__float_as_uint(__fmul_rn(rf, scale)) | s);
    if (e < 897u) { h = __uint_as_float(s); l = __uint_as_float(s); }
    else if (e > 1150u) { h = __uint_as_float(0x7fc00000u); l = 0.f; }
    else { h = __uint_as_float(hb); l = e < 949u ? __uint_as_float(s) : lf; }
}
__device__ __forceinline__ float d2f_bits(double x) {  // truncation to FP32 (same range rules)
    float h, l;
    d2ff_bits(x, h, l);
    return h;
}

// ---- double-FP32 ("float-float") arithmetic on packed FP32x2 lanes ----------------------------
// A value is an unevaluated sum h + l of two FP32 numbers (about 48 significant bits).  Products
// use the exact FMA residual (fma(a, b, -a*b) is the rounding error of a*b), sums the TwoSum
// error-free transformation; the absolute error of a sum or product is about 2^-46 of its largest
// operand.  Used by the first-order sweeps of chunks in supersonic flow, where the reference scheme
// amplifies per-step rounding errors (its split gives the u - a wave the negative numerical
// viscosity a(1 - M)/2 once M > 1), so that FP32 rounding is not enough there.
struct FF2 {
    float2 h, l;
};
__device__ __forceinline__ FF2 ffv(float h, float l) { return {f2(h), f2(l)}; }
__device__ __forceinline__ FF2 ffneg(FF2 a) { return {neg2(a.h), neg2(a.l)}; }
// a * s for a power of two s (exact)
__device__ __forceinline__ FF2 ffscale(FF2 a, float s) { return {mul2(a.h, f2(s)), mul2(a.l, f2(s))}; }
// renormalisation of p + e with |e| small against |p|
__device__ __forceinline__ FF2 ffnorm(float2 p, float2 e) {
    const float2 h = add2(p, e);
    return {h, sub2(e, sub2(h, p))};
}
// sum without the final renormalisation: (s, e) with e = the rounding error of the high parts plus
// the low parts; for sums that feed another sum or a product
__device__ __forceinline__ FF2 ffadd_u(FF2 a, FF2 b) {
    const float2 s = add2(a.h, b.h);
    const float2 bp = sub2(s, a.h);
    const float2 e = add2(sub2(a.h, sub2(s, bp)), sub2(b.h, bp));
    return {s, add2(e, add2(a.l, b.l))};
}
__device__ __forceinline__ FF2 ffadd(FF2 a, FF2 b) {
    const FF2 t = ffadd_u(a, b);
    return ffnorm(t.h, t.l);
}
__device__ __forceinline__ FF2 ffsub(FF2 a, FF2 b) { return ffadd(a, ffneg(b)); }
// product left unnormalised, (p, e) with |e| <= about 2^-22 |p|; for products that feed a sum or
// another product, which renormalise
__device__ __forceinline__ FF2 ffmul_u(FF2 a, FF2 b) {
    const float2 p = mul2(a.h, b.h);
    float2 e = fma2(a.h, b.h, neg2(p));
    e = fma2(a.h, b.l, e);
    return {p, fma2(a.l, b.h, e)};
}
__device__ __forceinline__ FF2 ffmul(FF2 a, FF2 b) {
    const FF2 t = ffmul_u(a, b);
    return ffnorm(t.h, t.l);
}
// 1/a: r0 = approximate FP32 reciprocal, e = 1 - a r0 (FMA residuals), r = r0 (1 + e + e^2)
__device__ __forceinline__ FF2 ffrcp(FF2 a) {
    const float2 r0 = rcp2(a.h);
    float2 e = fma2(neg2(a.h), r0, f2(1.0f));
    e = fma2(neg2(a.l), r0, e);
    return ffnorm(r0, mul2(r0, fma2(e, e, e)));
}
// sqrt(a), a > 0: FP32 estimate s0 from a Newton-refined reciprocal square root y, then
// s = s0 + (a - s0^2) y / 2 (the residual a - s0^2 from an FMA)
__device__ __forceinline__ FF2 ffsqrt(FF2 a) {
    float2 y = rsqrt2(a.h);
    y = mul2(y, fma2(mul2(f2(-0.5f), a.h), mul2(y, y), f2(1.5f)));
    const float2 s0 = mul2(a.h, y);
    const float2 e = add2(fma2(neg2(s0), s0, a.h), a.l);
    return ffnorm(s0, mul2(mul2(f2(0.5f), e), y));
}

// The split fluxes of two cells (FP32x2 lanes) with conserved state U (pairs), evaluated directly
// in double-FP32 arithmetic (base-c/base_shll.c:134-158 with P = (gamma-1)(E - m u / 2), which
// equals rho R T, and a^2 = gamma R T = gamma (gamma-1) (E - m u / 2) / rho).  Absolute errors are
// about 2^-45 of the flux magnitudes, so no deviation form is needed.  gg1 = gamma (gamma-1),
// gm1 = gamma - 1, as pairs.
__device__ __forceinline__ void flux1x2_ff(const FF2 U[3], FF2 gg1, FF2 gm1, FF2 fp[3], FF2 fm[3]) {
    const FF2 r = ffrcp(U[0]);
    const FF2 u = ffmul(U[1], r);
    const FF2 mu = ffmul_u(U[1], u);
    const FF2 eint = ffsub(U[2], ffscale(mu, 0.5f));
    const FF2 P = ffmul(gm1, eint);
    const FF2 a = ffsqrt(ffmul(gg1, ffmul_u(eint, r)));
    const FF2 M = ffmul(u, ffrcp(a));
    const FF2 Z1 = ffscale(ffadd(M, ffv(1.0f, 0.0f)), 0.5f);
    const FF2 Z2 = ffmul(ffscale(a, 0.5f), ffsub(ffv(1.0f, 0.0f), ffmul_u(M, M)));
    FF2 F[3];
    F[0] = U[1];
    F[1] = ffadd(mu, P);
    F[2] = ffmul(u, ffadd_u(U[2], P));
#pragma unroll
    for (int k = 0; k < 3; k++) {
        fp[k] = ffadd(ffmul_u(F[k], Z1), ffmul_u(U[k], Z2));
        fm[k] = ffsub(F[k], fp[k]);
    }
}

// minmod of two pairs per lane, as the reference's minmod (base-c/2nd_order_base_shll.c:191-201):
// 0 unless both have the same sign, else the one of smaller magnitude (the second on a tie); a
// pair's sign is that of its high part and magnitudes compare by high, then low parts
__device__ __forceinline__ float2 ffsel(bool q0, bool q1, float2 a, float2 b) {
    return make_float2(q0 ? a.x : b.x, q1 ? a.y : b.y);
}
__device__ __forceinline__ FF2 ffminmod(FF2 a, FF2 b) {
    bool pick_a[2], zero[2];
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const float ah = lane(a.h, q), al = lane(a.l, q), bh = lane(b.h, q), bl = lane(b.l, q);
        zero[q] = !((ah > 0.f && bh > 0.f) || (ah < 0.f && bh < 0.f));
        const float sa = ah < 0.f ? -1.f : 1.f, sb = bh < 0.f ? -1.f : 1.f;
        const float mah = fabsf(ah), mbh = fabsf(bh);
        pick_a[q] = mah < mbh || (mah == mbh && __fmul_rn(sa, al) < __fmul_rn(sb, bl));
    }
    FF2 r = {ffsel(pick_a[0], pick_a[1], a.h, b.h), ffsel(pick_a[0], pick_a[1], a.l, b.l)};
    r.h = ffsel(zero[0], zero[1], f2(0.f), r.h);
    r.l = ffsel(zero[0], zero[1], f2(0.f), r.l);
    return r;
}
// limited slope from the differences a = f_j - f_{j-1}, b = f_{j+1} - f_j: minmod (LIM = 0) or the
// MC limiter minmod((a+b)/2, alpha minmod(a, b)) (LIM = 1, base-omp/2nd_order_base_shll.c:316-325)
template <int LIM>
__device__ __forceinline__ FF2 ffslope(FF2 a, FF2 b, float alpha) {
    if (LIM == 1) return ffminmod(ffscale(ffadd(a, b), 0.5f), ffmul(ffv(alpha, 0.f), ffminmod(a, b)));
    return ffminmod(a, b);
}

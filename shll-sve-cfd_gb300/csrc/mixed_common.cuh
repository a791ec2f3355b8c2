// Device helpers of the mixed-precision engine: FP32-pair (compensated) arithmetic and the
// split fluxes of a cell evaluated in FP32 as deviations from an anchor state.
//
// Split fluxes (base-c/base_shll.c:134-158):  M = u/a, Z1 = (M+1)/2, Z2 = a(1-M^2)/2,
// Z3 = (M-1)/2 = Z1 - 1, P = rho R T, F = (m, m u + P, u (E + P)),
// fp = F Z1 + U Z2, fm = -F Z3 - U Z2.  Every quantity q is written as q* + dq with q* the
// anchor value; the deviations obey exact identities, e.g.
//   du = (dm - u* drho)/rho,  de = (dE - e* drho)/rho,  dT = (de - (u + u*) du / 2)/CV,
//   da = gamma R dT/(a + a*),  dM = (du - M* da)/a,  dZ2 = (da (1-M^2) - a* (M + M*) dM)/2,
//   dP = R (drho T + rho* dT),  dfp = dF Z1 + F* dZ1 + dU Z2 + U* dZ2,
//   dfm = -(dF Z3 + F* dZ1) - (dU Z2 + U* dZ2),
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

__device__ __forceinline__ float minmod_f(float l, float r) {
    if (__fmul_rn(l, r) < 0.f) return 0.f;
    return fabsf(l) < fabsf(r) ? l : r;
}
// limited slope from three consecutive values: minmod (LIM = 0), or the MC limiter (LIM = 1,
// base-omp/2nd_order_base_shll.c:316-325)
template <int LIM>
__device__ __forceinline__ float slope_f(float fl, float fc, float fr, float alpha) {
    float a = __fadd_rn(fc, -fl), b = __fadd_rn(fr, -fc);
    if (LIM == 1) return minmod_f(__fmul_rn(0.5f, __fadd_rn(fr, -fl)), __fmul_rn(alpha, minmod_f(a, b)));
    return minmod_f(a, b);
}

__device__ __forceinline__ float fast_rcp(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ float fast_sqrt(float x) { return __fmul_rn(x, rsqrtf(x)); }

// 1D split-flux deviations of a cell with conserved deviation d = (drho, dm, dE)
__device__ __forceinline__ void dflux1(const AnchorCoef& c, const float d[3], float dfp[3], float dfm[3]) {
    const float drho = d[0], dm = d[1], dE = d[2];
    const float rho = __fadd_rn(c.rho, drho);
    const float r = fast_rcp(rho);
    const float du = __fmul_rn(__fmaf_rn(-c.u, drho, dm), r);
    const float u = __fadd_rn(c.u, du);
    const float de = __fmul_rn(__fmaf_rn(-c.e, drho, dE), r);
    const float dT = __fmul_rn(__fmaf_rn(-0.5f * 1.0f, __fmul_rn(__fadd_rn(u, c.u), du), de), c.cvinv);
    const float T = __fadd_rn(c.T, dT);
    const float gRT = __fmul_rn(c.gR, T);
    const float ainv = rsqrtf(gRT);           // 1/a
    const float a = __fmul_rn(gRT, ainv);     // a = sqrt(gamma R T)
    const float da = __fmul_rn(__fmul_rn(c.gR, dT), fast_rcp(__fadd_rn(a, c.a)));
    const float dM = __fmul_rn(__fmaf_rn(-c.M, da, du), ainv);
    const float M = __fadd_rn(c.M, dM);
    const float dZ1 = __fmul_rn(0.5f, dM);
    const float Z1 = __fadd_rn(c.Z1, dZ1);
    const float Z3 = __fadd_rn(Z1, -1.0f);
    const float omm = __fmaf_rn(-M, M, 1.0f);
    const float dZ2 = __fmul_rn(0.5f, __fmaf_rn(da, omm, -__fmul_rn(__fmul_rn(c.a, __fadd_rn(M, c.M)), dM)));
    const float Z2 = __fadd_rn(c.Z2, dZ2);
    const float dP = __fmul_rn(c.R, __fmaf_rn(drho, T, __fmul_rn(c.rho, dT)));
    const float P = __fadd_rn(c.P, dP);
    const float E = __fadd_rn(c.Uf[2], dE);
    float dF[3];
    dF[0] = dm;
    dF[1] = __fadd_rn(__fmaf_rn(dm, u, __fmul_rn(c.Uf[1], du)), dP);
    dF[2] = __fmaf_rn(du, __fadd_rn(E, P), __fmul_rn(c.u, __fadd_rn(dE, dP)));
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const float a1 = __fmaf_rn(dF[k], Z1, __fmul_rn(c.F[k], dZ1));
        const float a2 = __fmaf_rn(d[k], Z2, __fmul_rn(c.Uf[k], dZ2));
        const float a3 = __fmaf_rn(dF[k], Z3, __fmul_rn(c.F[k], dZ1));
        dfp[k] = __fadd_rn(a1, a2);
        dfm[k] = -__fadd_rn(a3, a2);
    }
}

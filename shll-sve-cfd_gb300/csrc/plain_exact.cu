// SHLL_PREC_F64_EXACT and SHLL_PREC_F32_EXACT: reference arithmetic with every multiply and add
// rounded separately (this file is compiled with -fmad=false), IEEE division and square root:
// bit-identical to the reference's gcc builds (which contain no fused multiply-add on x86-64).
#define SHLL_PLAIN_NS plain_exact
#include "shll_plain.cuh"

namespace plain_exact {
cudaError_t step(const PlainArgs& a) { return a.real_bits == 32 ? step_t<float>(a) : step_t<double>(a); }
cudaError_t stage(const PlainArgs& a, int which) {
    return a.real_bits == 32 ? stage_t<float>(a, which) : stage_t<double>(a, which);
}
}

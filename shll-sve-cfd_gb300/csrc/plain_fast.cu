// SHLL_PREC_F64: reference arithmetic in FP64 with fused multiply-add allowed (compiled with
// the default -fmad=true).
#define SHLL_PLAIN_NS plain_fast
#include "shll_plain.cuh"

namespace plain_fast {
cudaError_t step(const PlainArgs& a) { return step_t<double>(a); }
cudaError_t stage(const PlainArgs& a, int which) { return stage_t<double>(a, which); }
}

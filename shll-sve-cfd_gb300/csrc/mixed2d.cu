// Mixed-precision 2D engine (placeholder until the 2D kernels land).
#include <cstdio>

#include "mixed.h"

MixedState* mixed2d_attach(MixedState* m, char* err, size_t len) {
    snprintf(err, len, "2D mixed precision is not built yet");
    return nullptr;
}
void mixed2d_detach(MixedState*) {}
int mixed2d_load(MixedState*, int, const double*, char* err, size_t len) {
    snprintf(err, len, "2D mixed precision is not built yet");
    return SHLL_ERR_UNSUPPORTED;
}
int mixed2d_run(MixedState*, long, char* err, size_t len) {
    snprintf(err, len, "2D mixed precision is not built yet");
    return SHLL_ERR_UNSUPPORTED;
}
int mixed2d_item_conserved(MixedState*, int, double*, char* err, size_t len) {
    snprintf(err, len, "2D mixed precision is not built yet");
    return SHLL_ERR_UNSUPPORTED;
}
int mixed2d_totals(MixedState*, int, double*, char* err, size_t len) {
    snprintf(err, len, "2D mixed precision is not built yet");
    return SHLL_ERR_UNSUPPORTED;
}

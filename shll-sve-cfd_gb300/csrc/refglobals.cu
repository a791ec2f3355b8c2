// The reference program's own globals, for the reference-named entry points on the default context
// (Allocate_and_Init_Memory, Compute_U_from_P, ...).  A reference solver keeps its problem in
// file-scope constants and its time step in globals that main() reads (base-c/base_shll.c:15-26,
// base-c/base_shll_2d.c:21-36, base-c/2nd_order_base_shll.c:29-44): C gives those external linkage,
// so a program that keeps them and takes the stage functions from this library still links.  The
// constants are read through weak references (null when the loading program does not define them);
// the step variables are weak definitions here, which the program's own variables of the same name
// interpose, so that Compute_U_from_P sets the DT that the program's `time += DT` loop reads.
#include "shll_internal.h"
#include "../../include/shll.h"

extern "C" {
extern const int N __attribute__((weak));
extern const int NX __attribute__((weak));
extern const int NY __attribute__((weak));
extern const float R __attribute__((weak));
extern const float GAMMA __attribute__((weak));
extern const float L __attribute__((weak));
extern const float H __attribute__((weak));
extern const float CFL __attribute__((weak));
extern const float TOTAL_TIME __attribute__((weak));
extern float* dhm0 __attribute__((weak));   // a slope array of the second-order solver only
__attribute__((weak)) float DT = 0.f;
__attribute__((weak)) float DT_ON_DX = 0.f;
__attribute__((weak)) float DT_ON_DY = 0.f;
}

// Fills p from the program's constants when it defines the reference's problem (N, R, GAMMA, CFL,
// L and TOTAL_TIME; NX, NY and H in 2D): 1D first order, 2D first order, or 2D second order where the
// program also has the second-order slope arrays; the reference's own initial data and its
// published float arithmetic.  Returns false (p untouched) otherwise.
bool shll_ref_program_params(shll_params* p) {
    if (!&N || !&R || !&GAMMA || !&CFL || !&L || !&TOTAL_TIME) return false;
    const bool two_d = &NX && &NY && &H;
    const int order = two_d && &dhm0 ? 2 : 1;
    shll_params q;
    shll_params_default(&q, two_d ? 2 : 1, order);
    q.nx = two_d ? NX : N;
    q.ny = two_d ? NY : 1;
    q.R = R;
    q.gamma = GAMMA;
    q.cfl = CFL;
    q.lx = L;
    q.ly = two_d ? H : 1.0;
    q.t_end = TOTAL_TIME;
    q.precision = SHLL_PREC_F32_EXACT;
    q.clock_f32 = 1;
    if (q.nx < 2 || (two_d && q.ny < 2)) return false;
    *p = q;
    return true;
}

// Compute_U_from_P's step globals (base_shll.c:82-84, base_shll_2d.c:133-136)
void shll_ref_set_step(double dt, double dtdx, double dtdy) {
    DT = (float)dt;
    DT_ON_DX = (float)dtdx;
    DT_ON_DY = (float)dtdy;
}

/*
 * Reference-style driver over the C-ABI: the time loop of base-c/base_shll.c:198-225 with the
 * reference's own stage names, now served by libshll_gb300 on the GPU.  Usage:
 *   shll_tube [cells] [order 1|2] [precision: f64 | f64_exact | f32_exact | mixed_f64 | mixed_kahan]
 * Writes results.dat in the reference's format and prints the step count as the reference does.
 * For the plain precisions it calls the four stages per step exactly as the reference's main();
 * for the mixed precisions (which have no separate stages) it runs the fused time loop.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "shll.h"

int main(int argc, char** argv) {
    int n = argc > 1 ? atoi(argv[1]) : 256;
    int order = argc > 2 ? atoi(argv[2]) : 1;
    const char* prec = argc > 3 ? argv[3] : "f64";
    shll_params p;
    shll_params_default(&p, 1, order);
    p.nx = n;
    if (!strcmp(prec, "f64_exact")) p.precision = SHLL_PREC_F64_EXACT;
    else if (!strcmp(prec, "f32_exact")) p.precision = SHLL_PREC_F32_EXACT;
    else if (!strcmp(prec, "mixed_f64")) p.precision = SHLL_PREC_MIXED_F64;
    else if (!strcmp(prec, "mixed_kahan")) p.precision = SHLL_PREC_MIXED_KAHAN;
    else p.precision = SHLL_PREC_F64;
    if (shll_ref_configure(&p) != SHLL_OK) return 1;
    long total = shll_steps_for(&p);
    int NO_STEPS = 0;
    Allocate_and_Init_Memory();
    if (!shll_ref_context()) return 1;
    if (p.precision <= SHLL_PREC_F32_EXACT) {
        Compute_U_from_P();
        Compute_P_from_U();
        while (NO_STEPS < total) {
            Compute_F_from_P();
            Update_U_from_F();
            Compute_P_from_U();
            NO_STEPS += 1;
        }
    } else {
        long steps = 0;
        if (shll_run(shll_ref_context(), &steps) != SHLL_OK) {
            fprintf(stderr, "run failed: %s\n", shll_last_error(shll_ref_context()));
            return 1;
        }
        NO_STEPS = (int)steps;
    }
    printf("Completed in %d steps\n", NO_STEPS);
    Save_Results();
    Free_Memory();
    return 0;
}

/*
 * Reference-style OpenMP driver over the C-ABI: the main() of base-omp/2nd_order_base_shll.c:615-653
 * (a team of threads, each calling every stage, a barrier per time step, float time += DT), with
 * the stages served by libshll_gb300_omp (one thread of the team runs each stage on the GPU; the
 * team waits at the stage's implicit barrier).  Usage:
 *   shll_omp [cells per side] [threads] [precision: f32_exact | f64_exact | f64] [steps]
 * Defaults follow base-omp: 1024 x 1024, 16 threads, second order, MC limiter alpha 1.25, the
 * quadrant initial data, t_end 0.3 (steps > 0 runs exactly that many steps instead).
 * Writes results.dat in the reference's format and prints the step count as the reference does.
 */
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "shll.h"

int shll_omp_status(void);  /* libshll_gb300_omp: first failing stage status, 0 if none */

int main(int argc, char** argv) {
    const int n = argc > 1 ? atoi(argv[1]) : 1024;
    const int threads = argc > 2 ? atoi(argv[2]) : 16;
    const char* prec = argc > 3 ? argv[3] : "f32_exact";
    const long nsteps = argc > 4 ? atol(argv[4]) : 0;
    shll_params p;
    shll_params_default(&p, 2, 2);
    p.nx = p.ny = n;
    p.limiter = 1;
    p.mc_alpha = 1.25;
    p.t_end = 0.3;
    p.n_steps = nsteps;
    p.ic.kind = SHLL_IC_QUADRANTS2D;
    if (!strcmp(prec, "f64_exact")) p.precision = SHLL_PREC_F64_EXACT;
    else if (!strcmp(prec, "f64")) p.precision = SHLL_PREC_F64;
    else p.precision = SHLL_PREC_F32_EXACT;
    p.clock_f32 = p.precision == SHLL_PREC_F32_EXACT;
    if (shll_ref_configure(&p) != SHLL_OK) return 1;
    Allocate_and_Init_Memory();
    if (!shll_ref_context()) return 1;
    const float DT = (float)shll_ref_dt();
    const float TOTAL_TIME = (float)p.t_end;

    omp_set_num_threads(threads);
#pragma omp parallel
    {
        int NO_STEPS = 0;
        Compute_U_from_P();
        Compute_P_from_U();
        float time = 0.0f;
        while (nsteps > 0 ? NO_STEPS < nsteps : time < TOTAL_TIME) {
            Compute_F_from_P();
            Update_U_from_F();
            Compute_P_from_U();
            time += DT;
            NO_STEPS += 1;
#pragma omp barrier
        }
#pragma omp master
        printf("Completed in %d steps (%d threads)\n", NO_STEPS, omp_get_num_threads());
    }
    Save_Results();
    Free_Memory();
    return shll_omp_status() != 0;
}

/*
 * The reference's stage functions with OpenMP team semantics, over the C-ABI of libshll_gb300.
 *
 * base-omp/2nd_order_base_shll.c:615-653 calls every stage from every thread of an OpenMP team;
 * inside, orphaned `omp for` loops share the cells among the threads and end in an implicit
 * barrier.  Here one thread of the team (`omp single`) runs the stage on the GPU (default context,
 * shll_ref_context()) and the others wait at the construct's implicit barrier, so the calling
 * pattern, the stage order and the synchronisation points are the reference's.  Called outside a
 * parallel region the functions behave like the serial shims of libshll_gb300.
 *
 * Linked ahead of libshll_gb300 (-lshll_gb300_omp -lshll_gb300), these definitions take the
 * place of the serial ones for the four stages that the reference calls inside its parallel
 * region; Allocate_and_Init_Memory, Save_Results and Free_Memory stay the serial ones.
 * A failing stage is reported on stderr and recorded (shll_omp_status), as the reference checks
 * no return values.
 */
#include <stdio.h>

#include "shll.h"

static int g_status = SHLL_OK;

/* first non-zero status of a team stage since the process started (0 if none) */
int shll_omp_status(void) { return g_status; }

static void report(int rc, const char* what) {
    if (rc == SHLL_OK) return;
    if (g_status == SHLL_OK) g_status = rc;
    shll_ctx* c = shll_ref_context();
    fprintf(stderr, "%s: %s (%s)\n", what, shll_status_string(rc), c ? shll_last_error(c) : "no context");
}

void Compute_U_from_P(void) {
#pragma omp single
    report(shll_compute_U_from_P(shll_ref_context()), "Compute_U_from_P");
}

void Compute_P_from_U(void) {
#pragma omp single
    report(shll_compute_P_from_U(shll_ref_context()), "Compute_P_from_U");
}

void Compute_F_from_P(void) {
#pragma omp single
    report(shll_compute_F_from_P(shll_ref_context()), "Compute_F_from_P");
}

void Update_U_from_F(void) {
#pragma omp single
    report(shll_update_U_from_F(shll_ref_context()), "Update_U_from_F");
}

/* A reference-style solver program linked against libshll_gb300.so with nothing changed in its main():
 * the structure of base-c/base_shll.c (its file-scope problem constants :15-26 and its time loop
 * :198-225 on its own float clock and DT global), with the stage functions taken from the library
 * instead of defined in this file.  The library reads the constants below (N, R, GAMMA, L, CFL,
 * TOTAL_TIME) to set up its default context in the reference's float arithmetic, and its
 * Compute_U_from_P sets DT and DT_ON_DX here, as the reference's own Compute_U_from_P does.
 * Output: "Completed in <steps> steps" and results.dat. */
#include <stdio.h>

#include "shll.h"

const int N = 1024;
const float R = 1.0;
const float GAMMA = 1.4;
const float L = 1.0;
const float CFL = 0.25;
float DT;
float DT_ON_DX;
int NO_STEPS = 0;
const float TOTAL_TIME = 0.2;

int main(void) {
    float time = 0.0;
    Allocate_and_Init_Memory();
    Compute_U_from_P();
    Compute_P_from_U();
    while (time < TOTAL_TIME) {
        Compute_F_from_P();
        Update_U_from_F();
        Compute_P_from_U();
        time += DT;
        NO_STEPS += 1;
    }
    printf("Completed in %d steps\n", NO_STEPS);
    Save_Results();
    Free_Memory();
    return 0;
}

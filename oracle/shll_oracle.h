/*
 * CPU oracle for the SHLL Euler hot path.  TEST INFRASTRUCTURE ONLY: this code is the
 * checker that the CUDA library is compared against.  Nothing in the product links it.
 *
 * It restates, operation by operation, the SHLL solvers of the reference project
 * (archembaud/shll-sve-cfd):
 *   base-c/base_shll.c           1D, first order, reflective walls
 *   base-c/2nd_order_base_shll.c 2D, second order (minmod on split fluxes), outflow walls;
 *                                its x sweep, restricted to 1D, is the 1D second-order scheme
 *   base-c/base_shll_2d.c        2D, first order, reflective walls
 *   base-omp/2nd_order_base_shll.c  MC limiter variant of the second-order slopes
 * in two arithmetic types:
 *   real_bits = 32: the reference as published (float arrays, with the double promotions that
 *                   its double literals and sqrt() cause, reproduced cast by cast);
 *   real_bits = 64: the reference with every float replaced by double.
 * Both reproduce the compiled reference bit for bit when built with -ffp-contract=off
 * (pinned by tests against binaries built from the reference sources).
 */
#ifndef SHLL_ORACLE_H
#define SHLL_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_cfg {
    int dim;          /* 1 or 2 */
    int order;        /* 1: first order, reflective walls; 2: second order, outflow walls */
    int nx, ny;       /* cells; ny = 1 in 1D.  2D cell index = i*ny + j (y contiguous) */
    int real_bits;    /* 32 or 64 */
    int limiter;      /* second order only: 0 minmod, 1 MC limiter with mc_alpha */
    double mc_alpha;
    double gamma, R, cfl, lx, ly;
    double t_end;     /* loop while time < t_end ... */
    long n_steps;     /* ... unless n_steps > 0, then exactly n_steps steps */
} oracle_cfg;

/* Runs the solver from primitive state prim_in (nvar planes of ncell doubles: rho, u, [v], T)
 * and writes the final primitives and conserved variables (rho, rho*u, [rho*v], E) as doubles.
 * Returns the number of steps taken, or -1 on a bad configuration. */
long oracle_run(const oracle_cfg* cfg, const double* prim_in, double* prim_out, double* cons_out);

/* One evaluation of the split fluxes from conserved state: P from U, then F from P.
 * fp, fm (and hp, hm in 2D) are nvar planes of ncell. */
int oracle_split_fluxes(const oracle_cfg* cfg, const double* cons, double* fp, double* fm,
                        double* hp, double* hm);

/* Threads of the stage loops (OpenMP builds; n <= 0: all processors); returns the count in use
 * (1 without OpenMP).  Results do not depend on it. */
int oracle_set_threads(int n);

/* Step count of the reference time loop (time += DT in the chosen type until time >= t_end). */
long oracle_count_steps(const oracle_cfg* cfg);

/* Initial conditions, written as primitive planes (double). */
void oracle_ic_sod(int n, double x_d, double rhoL, double uL, double TL,
                   double rhoR, double uR, double TR, double* prim);
void oracle_ic_ref_box2d(int nx, int ny, double* prim);       /* base_shll_2d.c:92-103 */
void oracle_ic_four_shock2d(int nx, int ny, int real_bits, double R, double* prim); /* 2nd_order:133-149 */
void oracle_ic_quadrants2d(int nx, int ny, int real_bits, double R, double* prim); /* base-omp/2nd_order_base_shll.c:147-172 */
void oracle_ic_circle2d(int nx, int ny, double lx, double ly, double cx, double cy, double r,
                        double rho_in, double T_in, double rho_out, double T_out, double* prim);

/* Exact solution of the 1D Riemann problem (Toro, Riemann Solvers and Numerical Methods for
 * Fluid Dynamics, ch. 4), sampled at cell centres x_i = (i+0.5)*dx at time t.  Pressure is
 * p = rho*R*T; the output is primitive planes rho, u, T. Returns Newton iterations or -1. */
int oracle_riemann_exact(double gamma, double R, double rhoL, double uL, double TL,
                         double rhoR, double uR, double TR, double x_d, double t,
                         int n, double lx, double* prim);

#ifdef __cplusplus
}
#endif
#endif

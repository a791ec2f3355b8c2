/*
 * CPU oracle for the SHLL Euler hot path -- TEST INFRASTRUCTURE ONLY (see shll_oracle.h).
 * Only tests/, the smoke check and the CPU-baseline leg of bench.py load this library.
 * Build with -O2 -ffp-contract=off so that no multiply-add is fused: the reference binaries
 * built by gcc -O3 on x86-64 contain no FMA, and the Arm build must not add any.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "shll_oracle.h"

/* Threads of the stage loops (base-omp/2nd_order_base_shll.c:615-653 runs the same stages with an
 * OpenMP team; every cell of a stage is computed independently of the others, so the results do
 * not depend on the thread count).  1 unless oracle_set_threads() asks for more. */
static int g_threads = 1;
#ifdef _OPENMP
#include <omp.h>
#define ORACLE_OMP_FOR _Pragma("omp parallel for if (g_threads > 1) num_threads(g_threads) schedule(static)")
#else
#define ORACLE_OMP_FOR
#endif

#define REAL float
#define SFX _f32
#include "shll_oracle_impl.h"
#undef REAL
#undef SFX

#define REAL double
#define SFX _f64
#include "shll_oracle_impl.h"
#undef REAL
#undef SFX

static int cfg_ok(const oracle_cfg* c) {
    if (!c) return 0;
    if (c->dim != 1 && c->dim != 2) return 0;
    if (c->order != 1 && c->order != 2) return 0;
    if (c->real_bits != 32 && c->real_bits != 64) return 0;
    if (c->nx < 2 || (c->dim == 2 && c->ny < 2)) return 0;
    if (c->limiter != 0 && c->limiter != 1) return 0;
    return 1;
}

long oracle_run(const oracle_cfg* c, const double* prim_in, double* prim_out, double* cons_out) {
    if (!cfg_ok(c) || !prim_in) return -1;
    return c->real_bits == 32 ? run_f32(c, prim_in, prim_out, cons_out)
                              : run_f64(c, prim_in, prim_out, cons_out);
}

int oracle_split_fluxes(const oracle_cfg* c, const double* cons, double* fp, double* fm,
                        double* hp, double* hm) {
    if (!cfg_ok(c) || !cons || !fp || !fm) return -1;
    return c->real_bits == 32 ? split_fluxes_f32(c, cons, fp, fm, hp, hm)
                              : split_fluxes_f64(c, cons, fp, fm, hp, hm);
}

long oracle_count_steps(const oracle_cfg* c) {
    if (!cfg_ok(c)) return -1;
    return c->real_bits == 32 ? count_steps_f32(c) : count_steps_f64(c);
}

/* base-c/base_shll.c:53-60: cells with i < x_d*N take the left state (the reference uses
 * x_d = 0.5 and compares in double). */
void oracle_ic_sod(int n, double x_d, double rhoL, double uL, double TL,
                   double rhoR, double uR, double TR, double* prim) {
    for (int i = 0; i < n; i++) {
        int left = i < x_d * n;
        prim[i] = left ? rhoL : rhoR;
        prim[n + i] = left ? uL : uR;
        prim[2 * n + i] = left ? TL : TR;
    }
}

/* base-c/base_shll_2d.c:92-103: rho = 1 strictly inside (0.2, 0.8)^2 in index space, else 10;
 * at rest, T = 1. */
void oracle_ic_ref_box2d(int nx, int ny, double* prim) {
    size_t n = (size_t)nx * ny;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            size_t c = (size_t)i * ny + j;
            int in = (i > 0.2 * nx) && (i < 0.8 * nx) && (j > 0.2 * ny) && (j < 0.8 * ny);
            prim[c] = in ? 1.0 : 10.0;
            prim[n + c] = 0.0;
            prim[2 * n + c] = 0.0;
            prim[3 * n + c] = 1.0;
        }
}

/* base-c/2nd_order_base_shll.c:133-149 (four-shock problem).  T = p/(rho R) is evaluated as the
 * reference does: rho*R in the reference's float (or double) type, then a double division. */
void oracle_ic_four_shock2d(int nx, int ny, int real_bits, double R, double* prim) {
    size_t n = (size_t)nx * ny;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            size_t c = (size_t)i * ny + j;
            double rho, u, v, pr;
            if ((i < 0.75 * nx) && (j < 0.75 * ny)) { rho = 0.138; u = 1.206; v = 1.206; pr = 0.029; }
            else if ((i > 0.75 * nx) && (j < 0.75 * ny)) { rho = 0.5323; u = 0.0; v = 1.206; pr = 0.3; }
            else if ((i < 0.75 * nx) && (j > 0.75 * ny)) { rho = 0.5323; u = 1.206; v = 0.0; pr = 0.3; }
            else { rho = 1.5; u = 0.0; v = 0.0; pr = 1.5; }
            double T;
            if (real_bits == 32) {
                float rf = (float)rho, Rf = (float)R;
                rho = rf; u = (float)u; v = (float)v;
                T = (float)(pr / (double)(rf * Rf));
            } else {
                T = pr / (rho * R);
            }
            prim[c] = rho; prim[n + c] = u; prim[2 * n + c] = v; prim[3 * n + c] = T;
        }
}

/* base-omp/2nd_order_base_shll.c:147-172 ("Configuration 6"): four quadrants at pressure 1;
 * T = 1/(rho R) with rho*R in the reference's type. */
void oracle_ic_quadrants2d(int nx, int ny, int real_bits, double R, double* prim) {
    size_t n = (size_t)nx * ny;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            size_t c = (size_t)i * ny + j;
            double rho, u, v;
            if ((i < 0.5 * nx) && (j < 0.5 * ny)) { rho = 1.0; u = -0.75; v = 0.5; }
            else if ((i > 0.5 * nx) && (j < 0.5 * ny)) { rho = 3.0; u = -0.75; v = -0.5; }
            else if ((i < 0.5 * nx) && (j > 0.5 * ny)) { rho = 2.0; u = 0.75; v = 0.5; }
            else { rho = 1.0; u = 0.75; v = -0.5; }
            double T = real_bits == 32 ? (double)(float)(1.0 / (double)((float)rho * (float)R)) : 1.0 / (rho * R);
            prim[c] = rho; prim[n + c] = u; prim[2 * n + c] = v; prim[3 * n + c] = T;
        }
}

/* Circular diaphragm: cell centres ((i+0.5) dx, (j+0.5) dy) strictly inside radius r. */
void oracle_ic_circle2d(int nx, int ny, double lx, double ly, double cx, double cy, double r,
                        double rho_in, double T_in, double rho_out, double T_out, double* prim) {
    size_t n = (size_t)nx * ny;
    double dx = lx / nx, dy = ly / ny;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            size_t c = (size_t)i * ny + j;
            double x = (i + 0.5) * dx - cx, y = (j + 0.5) * dy - cy;
            int in = x * x + y * y < r * r;
            prim[c] = in ? rho_in : rho_out;
            prim[n + c] = 0.0;
            prim[2 * n + c] = 0.0;
            prim[3 * n + c] = in ? T_in : T_out;
        }
}

/* ---- exact Riemann solver (Toro, ch. 4), written from the published equations ---- */
typedef struct { double rho, u, p, c; } rstate;

static void pressure_fn(double g, double p, const rstate* k, double* f, double* df) {
    if (p > k->p) {             /* shock branch */
        double A = 2.0 / ((g + 1.0) * k->rho), B = (g - 1.0) / (g + 1.0) * k->p;
        double q = sqrt(A / (B + p));
        *f = (p - k->p) * q;
        *df = q * (1.0 - 0.5 * (p - k->p) / (B + p));
    } else {                    /* rarefaction branch */
        double pr = p / k->p;
        *f = 2.0 * k->c / (g - 1.0) * (pow(pr, 0.5 * (g - 1.0) / g) - 1.0);
        *df = 1.0 / (k->rho * k->c) * pow(pr, -0.5 * (g + 1.0) / g);
    }
}

static void sample(double g, double ps, double us, const rstate* L, const rstate* Rr, double S,
                   double* rho, double* u, double* p) {
    double gm = (g - 1.0) / (g + 1.0);
    if (S <= us) {
        if (ps > L->p) {
            double SL = L->u - L->c * sqrt((g + 1.0) / (2.0 * g) * ps / L->p + (g - 1.0) / (2.0 * g));
            if (S <= SL) { *rho = L->rho; *u = L->u; *p = L->p; }
            else { *rho = L->rho * (ps / L->p + gm) / (gm * ps / L->p + 1.0); *u = us; *p = ps; }
        } else {
            double SHL = L->u - L->c, cs = L->c * pow(ps / L->p, 0.5 * (g - 1.0) / g), STL = us - cs;
            if (S <= SHL) { *rho = L->rho; *u = L->u; *p = L->p; }
            else if (S > STL) { *rho = L->rho * pow(ps / L->p, 1.0 / g); *u = us; *p = ps; }
            else {
                double b = 2.0 / (g + 1.0) + (g - 1.0) / ((g + 1.0) * L->c) * (L->u - S);
                *rho = L->rho * pow(b, 2.0 / (g - 1.0));
                *u = 2.0 / (g + 1.0) * (L->c + 0.5 * (g - 1.0) * L->u + S);
                *p = L->p * pow(b, 2.0 * g / (g - 1.0));
            }
        }
    } else {
        if (ps > Rr->p) {
            double SR = Rr->u + Rr->c * sqrt((g + 1.0) / (2.0 * g) * ps / Rr->p + (g - 1.0) / (2.0 * g));
            if (S >= SR) { *rho = Rr->rho; *u = Rr->u; *p = Rr->p; }
            else { *rho = Rr->rho * (ps / Rr->p + gm) / (gm * ps / Rr->p + 1.0); *u = us; *p = ps; }
        } else {
            double SHR = Rr->u + Rr->c, cs = Rr->c * pow(ps / Rr->p, 0.5 * (g - 1.0) / g), STR = us + cs;
            if (S >= SHR) { *rho = Rr->rho; *u = Rr->u; *p = Rr->p; }
            else if (S <= STR) { *rho = Rr->rho * pow(ps / Rr->p, 1.0 / g); *u = us; *p = ps; }
            else {
                double b = 2.0 / (g + 1.0) - (g - 1.0) / ((g + 1.0) * Rr->c) * (Rr->u - S);
                *rho = Rr->rho * pow(b, 2.0 / (g - 1.0));
                *u = 2.0 / (g + 1.0) * (-Rr->c + 0.5 * (g - 1.0) * Rr->u + S);
                *p = Rr->p * pow(b, 2.0 * g / (g - 1.0));
            }
        }
    }
}

int oracle_riemann_exact(double g, double R, double rhoL, double uL, double TL,
                         double rhoR, double uR, double TR, double x_d, double t,
                         int n, double lx, double* prim) {
    rstate L = {rhoL, uL, rhoL * R * TL, 0}, Rr = {rhoR, uR, rhoR * R * TR, 0};
    L.c = sqrt(g * L.p / L.rho);
    Rr.c = sqrt(g * Rr.p / Rr.rho);
    if (2.0 / (g - 1.0) * (L.c + Rr.c) <= uR - uL) return -1;  /* vacuum is generated */
    double p = 0.5 * (L.p + Rr.p) - 0.125 * (uR - uL) * (L.rho + Rr.rho) * (L.c + Rr.c);
    if (p < 1e-8) p = 1e-8;
    int it;
    for (it = 1; it <= 100; it++) {
        double fL, dfL, fR, dfR;
        pressure_fn(g, p, &L, &fL, &dfL);
        pressure_fn(g, p, &Rr, &fR, &dfR);
        double pn = p - (fL + fR + uR - uL) / (dfL + dfR);
        if (pn < 1e-12) pn = 1e-12;
        double change = fabs(pn - p) / (0.5 * (pn + p));
        p = pn;
        if (change < 1e-15) break;
    }
    double fL, dfL, fR, dfR;
    pressure_fn(g, p, &L, &fL, &dfL);
    pressure_fn(g, p, &Rr, &fR, &dfR);
    double us = 0.5 * (uL + uR) + 0.5 * (fR - fL);
    double dx = lx / n;
    for (int i = 0; i < n; i++) {
        double x = (i + 0.5) * dx, rho, u, pr;
        double S = t > 0 ? (x - x_d) / t : (x < x_d ? -INFINITY : INFINITY);
        sample(g, p, us, &L, &Rr, S, &rho, &u, &pr);
        prim[i] = rho; prim[n + i] = u; prim[2 * n + i] = pr / (rho * R);
    }
    return it;
}

int oracle_set_threads(int n) {
#ifdef _OPENMP
    g_threads = n > 0 ? n : omp_get_num_procs();
#else
    (void)n;
    g_threads = 1;
#endif
    return g_threads;
}

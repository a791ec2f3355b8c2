/*
 * Type-generic body of the CPU oracle (TEST INFRASTRUCTURE ONLY).  Included twice by
 * shll_oracle.c, with REAL = float / SFX = _f32 and REAL = double / SFX = _f64.
 *
 * Every expression reproduces the evaluation order and the type promotions of the reference
 * C sources: D(x) marks an operand that the reference promotes to double because a double
 * literal (0.5, 1.0) or sqrt() touches it.  With REAL = double every D() is a no-op and the
 * code is the reference with float replaced by double.
 */
#define O_CAT2(a, b) a##b
#define O_CAT(a, b) O_CAT2(a, b)
#define FN(x) O_CAT(x, SFX)
#define D(x) ((double)(x))

typedef struct {
    int nx, ny, n, nv, dim, order, limiter;
    REAL *p[4], *u[4], *a;
    REAL *fp[4], *fm[4], *hp[4], *hm[4];
    REAL *dfp[4], *dfm[4], *dhp[4], *dhm[4];
    REAL R, GAMMA, CV, L, H, DX, DY, CFL, DT, DT_ON_DX, DT_ON_DY, TOTAL_TIME, alpha;
} FN(ost);

static void FN(ost_free)(FN(ost)* s) {
    for (int k = 0; k < 4; k++) {
        free(s->p[k]); free(s->u[k]); free(s->fp[k]); free(s->fm[k]); free(s->hp[k]); free(s->hm[k]);
        free(s->dfp[k]); free(s->dfm[k]); free(s->dhp[k]); free(s->dhm[k]);
    }
    free(s->a);
}

/* Constants exactly as the reference's file-scope const initialisers compute them
 * (base-c/base_shll.c:16-26, base-c/base_shll_2d.c:21-35). */
static int FN(ost_init)(FN(ost)* s, const oracle_cfg* c) {
    memset(s, 0, sizeof(*s));
    s->dim = c->dim; s->order = c->order; s->limiter = c->limiter;
    s->nx = c->nx; s->ny = (c->dim == 2) ? c->ny : 1; s->n = s->nx * s->ny;
    s->nv = (c->dim == 2) ? 4 : 3;
    s->R = (REAL)c->R;
    s->GAMMA = (REAL)c->gamma;
    s->CV = (REAL)(D(s->R) / (D(s->GAMMA) - 1.0));
    s->L = (REAL)c->lx;
    s->H = (REAL)c->ly;
    s->DX = s->L / (REAL)s->nx;
    s->DY = s->H / (REAL)s->ny;
    s->CFL = (REAL)c->cfl;
    s->TOTAL_TIME = (REAL)c->t_end;
    s->alpha = (REAL)c->mc_alpha;
    /* Compute_U_from_P: base-c/base_shll.c:83-84, base-c/base_shll_2d.c:134-136 */
    s->DT = (s->CFL / (s->R + 1)) * s->DX;
    s->DT_ON_DX = (s->CFL / (s->R + 1));
    s->DT_ON_DY = s->DT / s->DY;
    size_t bytes = (size_t)s->n * sizeof(REAL);
    for (int k = 0; k < s->nv; k++) {
        s->p[k] = calloc(1, bytes); s->u[k] = calloc(1, bytes);
        s->fp[k] = calloc(1, bytes); s->fm[k] = calloc(1, bytes);
        if (!s->p[k] || !s->u[k] || !s->fp[k] || !s->fm[k]) return -1;
        if (s->dim == 2) {
            s->hp[k] = calloc(1, bytes); s->hm[k] = calloc(1, bytes);
            if (!s->hp[k] || !s->hm[k]) return -1;
        }
        if (s->order == 2) {
            s->dfp[k] = calloc(1, bytes); s->dfm[k] = calloc(1, bytes);
            if (!s->dfp[k] || !s->dfm[k]) return -1;
            if (s->dim == 2) {
                s->dhp[k] = calloc(1, bytes); s->dhm[k] = calloc(1, bytes);
                if (!s->dhp[k] || !s->dhm[k]) return -1;
            }
        }
    }
    s->a = calloc(1, bytes);
    return s->a ? 0 : -1;
}

/* base-c/base_shll.c:74-80 (1D); base-c/base_shll_2d.c:124-131 (2D) */
static void FN(compute_U_from_P)(FN(ost)* s) {
    REAL **p = s->p, **u = s->u;
    for (int c = 0; c < s->n; c++) {
        if (s->dim == 1) {
            u[0][c] = p[0][c];
            u[1][c] = p[0][c] * p[1][c];
            u[2][c] = (REAL)(D(p[0][c]) * (D(p[2][c] * s->CV) + 0.5 * D(p[1][c]) * D(p[1][c])));
        } else {
            u[0][c] = p[0][c];
            u[1][c] = p[0][c] * p[1][c];
            u[2][c] = p[0][c] * p[2][c];
            u[3][c] = (REAL)(D(p[0][c]) * (D(p[3][c] * s->CV) + 0.5 * D(p[1][c] * p[1][c] + p[2][c] * p[2][c])));
        }
    }
}

/* base-c/base_shll.c:161-177 (1D); base-c/base_shll_2d.c:302-319 (2D) */
static void FN(compute_P_from_U)(FN(ost)* s) {
    REAL **p = s->p, **u = s->u;
    ORACLE_OMP_FOR
    for (int c = 0; c < s->n; c++) {
        p[0][c] = u[0][c];
        p[1][c] = u[1][c] / u[0][c];
        if (s->dim == 1) {
            p[2][c] = (REAL)((D(u[2][c] / u[0][c]) - 0.5 * D(p[1][c]) * D(p[1][c])) / D(s->CV));
            s->a[c] = (REAL)sqrt(D(s->GAMMA * s->R * p[2][c]));
        } else {
            p[2][c] = u[2][c] / u[0][c];
            p[3][c] = (REAL)((D(u[3][c] / u[0][c]) - 0.5 * D(p[1][c] * p[1][c] + p[2][c] * p[2][c])) / D(s->CV));
            s->a[c] = (REAL)sqrt(D(s->GAMMA * s->R * p[3][c]));
        }
    }
}

/* base-c/base_shll.c:130-159 (1D); base-c/base_shll_2d.c:239-300 (2D) */
static void FN(compute_F_from_P)(FN(ost)* s) {
    REAL **p = s->p, **u = s->u;
    ORACLE_OMP_FOR
    for (int c = 0; c < s->n; c++) {
        REAL Z1, Z2, Z3, M, P, f[4], h[4];
        if (s->dim == 1) {
            M = p[1][c] / s->a[c];
            Z1 = (REAL)(0.5 * (D(M) + 1.0));
            Z2 = (REAL)(0.5 * D(s->a[c]) * (1.0 - D(M * M)));
            Z3 = (REAL)(0.5 * (D(M) - 1.0));
            P = p[0][c] * s->R * p[2][c];
            f[0] = u[1][c];
            f[1] = u[1][c] * p[1][c] + P;
            f[2] = p[1][c] * (u[2][c] + P);
            for (int k = 0; k < 3; k++) {
                s->fp[k][c] = f[k] * Z1 + u[k][c] * Z2;
                s->fm[k][c] = -f[k] * Z3 - u[k][c] * Z2;
            }
        } else {
            P = p[0][c] * s->R * p[3][c];
            M = p[1][c] / s->a[c];
            Z1 = (REAL)(0.5 * (D(M) + 1.0));
            Z2 = (REAL)(0.5 * D(s->a[c]) * (1.0 - D(M * M)));
            Z3 = (REAL)(0.5 * (D(M) - 1.0));
            f[0] = u[1][c];
            f[1] = u[1][c] * p[1][c] + P;
            f[2] = u[1][c] * p[2][c];
            f[3] = p[1][c] * (u[3][c] + P);
            for (int k = 0; k < 4; k++) {
                s->fp[k][c] = f[k] * Z1 + u[k][c] * Z2;
                s->fm[k][c] = -f[k] * Z3 - u[k][c] * Z2;
            }
            M = p[2][c] / s->a[c];
            Z1 = (REAL)(0.5 * (D(M) + 1.0));
            Z2 = (REAL)(0.5 * D(s->a[c]) * (1.0 - D(M * M)));
            Z3 = (REAL)(0.5 * (D(M) - 1.0));
            h[0] = u[2][c];
            h[1] = u[2][c] * p[1][c];
            h[2] = u[2][c] * p[2][c] + P;
            h[3] = p[2][c] * (u[3][c] + P);
            for (int k = 0; k < 4; k++) {
                s->hp[k][c] = h[k] * Z1 + u[k][c] * Z2;
                s->hm[k][c] = -h[k] * Z3 - u[k][c] * Z2;
            }
        }
    }
}

/* base-c/2nd_order_base_shll.c:191-201 */
static REAL FN(minmod)(REAL left, REAL right) {
    if (left * right < 0.0) return (REAL)0.0;
    if (fabs(D(left)) < fabs(D(right))) return left;
    return right;
}

/* Slope of a split flux at an interior cell: minmod (2nd_order_base_shll.c:268-276) or the MC
 * limiter of base-omp/2nd_order_base_shll.c:316-325. */
static REAL FN(slope)(const FN(ost)* s, const REAL* f, int i, int st) {
    if (s->limiter == 1)
        return FN(minmod)((REAL)(0.5 * D(f[i + st] - f[i - st])),
                          s->alpha * FN(minmod)(f[i] - f[i - st], f[i + st] - f[i]));
    return FN(minmod)(f[i] - f[i - st], f[i + st] - f[i]);
}

/* First-order update with reflective walls: base-c/base_shll.c:87-128 (1D),
 * base-c/base_shll_2d.c:139-237 (2D: walls flip components 0,2,3 in x and 0,1,3 in y; the
 * x update is applied before the y update). */
static void FN(update_o1)(FN(ost)* s) {
    const int nx = s->nx, ny = s->ny, nv = s->nv;
    REAL **fp = s->fp, **fm = s->fm, **hp = s->hp, **hm = s->hm, **u = s->u;
    /* sign flips of the reflected split flux, per component */
    const REAL sx1[3] = {-1, 1, -1}, sx2[4] = {-1, 1, -1, -1}, sy2[4] = {-1, -1, 1, -1};
    const REAL* sx = (s->dim == 1) ? sx1 : sx2;
    ORACLE_OMP_FOR
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < ny; j++) {
            REAL Lf[4], Rf[4], Bf[4], Tf[4];
            int idx = i * ny + j;
            for (int k = 0; k < nv; k++) {
                if (i == 0) { Lf[k] = sx[k] * fm[k][idx]; Rf[k] = fm[k][idx + ny]; }
                else if (i == nx - 1) { Lf[k] = fp[k][idx - ny]; Rf[k] = sx[k] * fp[k][idx]; }
                else { Lf[k] = fp[k][idx - ny]; Rf[k] = fm[k][idx + ny]; }
                if (s->dim == 2) {
                    if (j == 0) { Bf[k] = sy2[k] * hm[k][idx]; Tf[k] = hm[k][idx + 1]; }
                    else if (j == ny - 1) { Bf[k] = hp[k][idx - 1]; Tf[k] = sy2[k] * hp[k][idx]; }
                    else { Bf[k] = hp[k][idx - 1]; Tf[k] = hm[k][idx + 1]; }
                }
            }
            /* the reference fills all Left/Right arrays before it updates any cell, and the
             * update of cell idx reads only cell idx's own Left/Right: updating in place here
             * is equivalent because fp/fm are not modified by the update. */
            for (int k = 0; k < nv; k++) {
                u[k][idx] = u[k][idx] - s->DT_ON_DX * (fp[k][idx] - fm[k][idx] + Rf[k] - Lf[k]);
                if (s->dim == 2)
                    u[k][idx] = u[k][idx] - s->DT_ON_DY * (hp[k][idx] - hm[k][idx] + Tf[k] - Bf[k]);
            }
        }
    }
}

/* Second-order update with outflow walls: base-c/2nd_order_base_shll.c:203-459.  Slopes of
 * the split fluxes (zero on edge cells), neighbour slopes (zero beyond the walls), then
 * U -= dt/dx (fp - fm + R - L) followed by U -= 0.5 dt/dx (dfp + dfm - Rdf - Ldf), and the same
 * in y for 2D.  In 1D this is the x sweep of that file. */
static void FN(update_o2)(FN(ost)* s) {
    const int nx = s->nx, ny = s->ny, nv = s->nv, n = s->n;
    REAL **fp = s->fp, **fm = s->fm, **hp = s->hp, **hm = s->hm, **u = s->u;
    /* slopes */
    ORACLE_OMP_FOR
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < ny; j++) {
            int idx = i * ny + j;
            for (int k = 0; k < nv; k++) {
                if (i == 0 || i == nx - 1) { s->dfp[k][idx] = 0; s->dfm[k][idx] = 0; }
                else {
                    s->dfp[k][idx] = FN(slope)(s, fp[k], idx, ny);
                    s->dfm[k][idx] = FN(slope)(s, fm[k], idx, ny);
                }
                if (s->dim == 2) {
                    if (j == 0 || j == ny - 1) { s->dhp[k][idx] = 0; s->dhm[k][idx] = 0; }
                    else {
                        s->dhp[k][idx] = FN(slope)(s, hp[k], idx, 1);
                        s->dhm[k][idx] = FN(slope)(s, hm[k], idx, 1);
                    }
                }
            }
        }
    }
    (void)n;
    /* gather + update (each cell reads only neighbours' fluxes and slopes, never neighbours' U) */
    ORACLE_OMP_FOR
    for (int i = 0; i < nx; i++) {
        for (int j = 0; j < ny; j++) {
            int idx = i * ny + j;
            for (int k = 0; k < nv; k++) {
                REAL Lf, Rf, Ldf, Rdf;
                if (i == 0) { Lf = fp[k][idx]; Rf = fm[k][idx + ny]; Ldf = 0; Rdf = s->dfm[k][idx + ny]; }
                else if (i == nx - 1) { Lf = fp[k][idx - ny]; Rf = fm[k][idx]; Ldf = s->dfp[k][idx - ny]; Rdf = 0; }
                else { Lf = fp[k][idx - ny]; Rf = fm[k][idx + ny]; Ldf = s->dfp[k][idx - ny]; Rdf = s->dfm[k][idx + ny]; }
                u[k][idx] = u[k][idx] - s->DT_ON_DX * (fp[k][idx] - fm[k][idx] + Rf - Lf);
                u[k][idx] = (REAL)(D(u[k][idx]) - 0.5 * D(s->DT_ON_DX) *
                                   D(s->dfp[k][idx] + s->dfm[k][idx] - Rdf - Ldf));
                if (s->dim == 2) {
                    REAL Bf, Tf, Bdf, Tdf;
                    if (j == 0) { Bf = hp[k][idx]; Tf = hm[k][idx + 1]; Bdf = 0; Tdf = s->dhm[k][idx + 1]; }
                    else if (j == ny - 1) { Bf = hp[k][idx - 1]; Tf = hm[k][idx]; Bdf = s->dhp[k][idx - 1]; Tdf = 0; }
                    else { Bf = hp[k][idx - 1]; Tf = hm[k][idx + 1]; Bdf = s->dhp[k][idx - 1]; Tdf = s->dhm[k][idx + 1]; }
                    u[k][idx] = u[k][idx] - s->DT_ON_DY * (hp[k][idx] - hm[k][idx] + Tf - Bf);
                    u[k][idx] = (REAL)(D(u[k][idx]) - 0.5 * D(s->DT_ON_DY) *
                                       D(s->dhp[k][idx] + s->dhm[k][idx] - Tdf - Bdf));
                }
            }
        }
    }
}

static void FN(load_prim)(FN(ost)* s, const double* prim) {
    for (int k = 0; k < s->nv; k++)
        for (int c = 0; c < s->n; c++) s->p[k][c] = (REAL)prim[(size_t)k * s->n + c];
}

static void FN(store)(const FN(ost)* s, double* prim, double* cons) {
    for (int k = 0; k < s->nv; k++)
        for (int c = 0; c < s->n; c++) {
            if (prim) prim[(size_t)k * s->n + c] = (double)s->p[k][c];
            if (cons) cons[(size_t)k * s->n + c] = (double)s->u[k][c];
        }
}

/* main(): base-c/base_shll.c:198-225 -- U from P, P from U, then
 * while (time < TOTAL_TIME) { F from P; update U; P from U; time += DT; } */
static long FN(run)(const oracle_cfg* c, const double* prim_in, double* prim_out, double* cons_out) {
    FN(ost) s;
    if (FN(ost_init)(&s, c) != 0) { FN(ost_free)(&s); return -1; }
    FN(load_prim)(&s, prim_in);
    FN(compute_U_from_P)(&s);
    FN(compute_P_from_U)(&s);
    long steps = 0;
    REAL time = 0;
    while (c->n_steps > 0 ? steps < c->n_steps : time < s.TOTAL_TIME) {
        FN(compute_F_from_P)(&s);
        if (s.order == 2) FN(update_o2)(&s); else FN(update_o1)(&s);
        FN(compute_P_from_U)(&s);
        time += s.DT;
        steps += 1;
    }
    FN(store)(&s, prim_out, cons_out);
    FN(ost_free)(&s);
    return steps;
}

static int FN(split_fluxes)(const oracle_cfg* c, const double* cons, double* fp, double* fm,
                            double* hp, double* hm) {
    FN(ost) s;
    if (FN(ost_init)(&s, c) != 0) { FN(ost_free)(&s); return -1; }
    for (int k = 0; k < s.nv; k++)
        for (int i = 0; i < s.n; i++) s.u[k][i] = (REAL)cons[(size_t)k * s.n + i];
    FN(compute_P_from_U)(&s);
    FN(compute_F_from_P)(&s);
    for (int k = 0; k < s.nv; k++)
        for (int i = 0; i < s.n; i++) {
            fp[(size_t)k * s.n + i] = s.fp[k][i];
            fm[(size_t)k * s.n + i] = s.fm[k][i];
            if (s.dim == 2 && hp && hm) {
                hp[(size_t)k * s.n + i] = s.hp[k][i];
                hm[(size_t)k * s.n + i] = s.hm[k][i];
            }
        }
    FN(ost_free)(&s);
    return 0;
}

static long FN(count_steps)(const oracle_cfg* c) {
    if (c->n_steps > 0) return c->n_steps;
    REAL R = (REAL)c->R, CFL = (REAL)c->cfl, L = (REAL)c->lx;
    REAL DX = L / (REAL)c->nx;
    REAL DT = (CFL / (R + 1)) * DX, TOTAL_TIME = (REAL)c->t_end, time = 0;
    long steps = 0;
    while (time < TOTAL_TIME) { time += DT; steps++; }
    return steps;
}

#undef FN
#undef D

// C-ABI of libshll_gb300 (include/shll.h): contexts, the reference's stages, fused stepping,
// results, and the reference's own entry-point names on a default context.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/shll.h"
#include "mixed.h"
#include "plain_batch.h"
#include "shll_internal.h"

struct shll_ctx {
    shll_params p;
    int n = 0, nv = 0, real_bits = 64;
    bool plain = true;             // plain (reference-arithmetic) kernels vs mixed engine
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // the reference's REAL-typed constants, widened to double
    double R = 0, GAMMA = 0, CV = 0, DX = 0, DY = 0, DT = 0, DT_ON_DX = 0, DT_ON_DY = 0;
    long steps_total = 0, steps_taken = 0;
    // plain state
    void* U[2] = {nullptr, nullptr};
    int cur = 0;
    void* P = nullptr;
    void* F[4] = {nullptr, nullptr, nullptr, nullptr};  // fp, fm, hp, hm (staged; lazily allocated)
    bool fluxes_valid = false;
    // device checkpoint of the plain state
    void* ckU = nullptr;
    void* ckP = nullptr;
    long ck_steps = -1;
    int ck_cur = 0;
    // mixed state
    MixedState* mixed = nullptr;
    int* d_flag = nullptr;
    bool initialized = false;
    char err[512] = {0};
};

static void set_err(shll_ctx* c, const char* fmt, ...) {
    if (!c) return;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(c->err, sizeof(c->err), fmt, ap);
    va_end(ap);
}

#define CUDA_TRY(ctx, call)                                                                        \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) {                                                                   \
            set_err(ctx, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return SHLL_ERR_CUDA;                                                                  \
        }                                                                                          \
    } while (0)

// ---------------- parameters ----------------
extern "C" void shll_params_default(shll_params* p, int dim, int order) {
    if (!p) return;
    memset(p, 0, sizeof(*p));
    p->dim = dim == 2 ? 2 : 1;
    p->order = order == 2 ? 2 : 1;
    p->nx = 256;
    p->ny = p->dim == 2 ? 256 : 1;
    p->gamma = 1.4;
    p->R = 1.0;
    p->cfl = 0.25;
    p->lx = 1.0;
    p->ly = 1.0;
    // base_shll.c:26, base_shll_2d.c:35, 2nd_order_base_shll.c:43
    p->t_end = p->dim == 1 ? 0.2 : (p->order == 1 ? 0.1 : 0.8);
    p->n_steps = 0;
    p->precision = SHLL_PREC_F64;
    p->limiter = 0;
    p->mc_alpha = 1.25;
    p->fold_steps = 0;
    p->clock_f32 = 0;
    if (p->dim == 1) {
        p->ic.kind = SHLL_IC_SOD;
        p->ic.x_d = 0.5;
        p->ic.rho_l = 10.0; p->ic.u_l = 0.0; p->ic.T_l = 1.0;
        p->ic.rho_r = 1.0; p->ic.u_r = 0.0; p->ic.T_r = 1.0;
    } else {
        p->ic.kind = p->order == 1 ? SHLL_IC_REF_BOX2D : SHLL_IC_FOUR_SHOCK2D;
    }
}

int shll_validate_params(const shll_params* p, char* err, size_t len) {
    if (!p) { snprintf(err, len, "params is NULL"); return SHLL_ERR_ARG; }
    if (p->dim != 1 && p->dim != 2) { snprintf(err, len, "dim must be 1 or 2 (got %d)", p->dim); return SHLL_ERR_ARG; }
    if (p->order != 1 && p->order != 2) { snprintf(err, len, "order must be 1 or 2 (got %d)", p->order); return SHLL_ERR_ARG; }
    if (p->nx < 2 || (p->dim == 2 && p->ny < 2)) { snprintf(err, len, "need nx, ny >= 2"); return SHLL_ERR_ARG; }
    long long cells = (long long)p->nx * (p->dim == 2 ? p->ny : 1);
    if (cells > (1LL << 30)) { snprintf(err, len, "too many cells (%lld > 2^30)", cells); return SHLL_ERR_ARG; }
    if (!(p->gamma > 1.0) || !(p->R > 0.0) || !(p->cfl > 0.0) || !(p->lx > 0.0) || (p->dim == 2 && !(p->ly > 0.0))) {
        snprintf(err, len, "need gamma > 1, R > 0, cfl > 0, lengths > 0");
        return SHLL_ERR_ARG;
    }
    if (p->n_steps <= 0 && !(p->t_end > 0.0)) { snprintf(err, len, "need t_end > 0 or n_steps > 0"); return SHLL_ERR_ARG; }
    if (p->precision < SHLL_PREC_F64 || p->precision > SHLL_PREC_MIXED_KAHAN) {
        snprintf(err, len, "unknown precision %d", p->precision);
        return SHLL_ERR_ARG;
    }
    if (p->limiter != 0 && p->limiter != 1) { snprintf(err, len, "limiter must be 0 or 1"); return SHLL_ERR_ARG; }
    if (p->order == 2 && p->limiter == 1 && !(p->mc_alpha > 0.0 && p->mc_alpha <= 2.0)) {
        snprintf(err, len, "MC limiter alpha must lie in (0, 2] (got %g)", p->mc_alpha);
        return SHLL_ERR_ARG;
    }
    if (p->fold_steps < 0) { snprintf(err, len, "fold_steps must be >= 0"); return SHLL_ERR_ARG; }
    int k = p->ic.kind;
    if (k < SHLL_IC_SOD || k > SHLL_IC_QUADRANTS2D) { snprintf(err, len, "unknown initial condition %d", k); return SHLL_ERR_ARG; }
    if (p->dim == 1 && k != SHLL_IC_SOD && k != SHLL_IC_USER) { snprintf(err, len, "initial condition %d is 2D only", k); return SHLL_ERR_ARG; }
    if (p->dim == 2 && k == SHLL_IC_SOD) { snprintf(err, len, "SOD initial condition is 1D only"); return SHLL_ERR_ARG; }
    if (k == SHLL_IC_SOD && (!(p->ic.rho_l > 0) || !(p->ic.rho_r > 0) || !(p->ic.T_l > 0) || !(p->ic.T_r > 0))) {
        snprintf(err, len, "initial densities and temperatures must be positive");
        return SHLL_ERR_ARG;
    }
    return SHLL_OK;
}

// The reference's const initialisers in its REAL type (base-c/base_shll.c:17-26, :83-84;
// base-c/base_shll_2d.c:24-35, :134-136).
template <typename REAL>
static void ref_constants(const shll_params* p, double* R, double* GAMMA, double* CV, double* DX, double* DY,
                          double* DT, double* DTDX, double* DTDY) {
    REAL r = (REAL)p->R, g = (REAL)p->gamma, cfl = (REAL)p->cfl, L = (REAL)p->lx, H = (REAL)p->ly;
    REAL cv = (REAL)((double)r / ((double)g - 1.0));
    REAL dx = L / (REAL)p->nx;
    REAL dy = H / (REAL)(p->dim == 2 ? p->ny : 1);
    REAL dt = (cfl / (r + 1)) * dx;
    REAL dtdx = cfl / (r + 1);
    REAL dtdy = dt / dy;
    *R = r; *GAMMA = g; *CV = cv; *DX = dx; *DY = dy; *DT = dt; *DTDX = dtdx; *DTDY = dtdy;
}

static int clock_is_f32(const shll_params* p) {
    return p->clock_f32 || p->precision == SHLL_PREC_F32_EXACT;
}

template <typename REAL>
static long count_steps_t(const shll_params* p) {
    double R, G, CV, DX, DY, DT, a, b;
    ref_constants<REAL>(p, &R, &G, &CV, &DX, &DY, &DT, &a, &b);
    REAL dt = (REAL)DT, t_end = (REAL)p->t_end, time = 0;
    long steps = 0;
    while (time < t_end) {
        time += dt;
        steps++;
        if (steps > (1L << 40)) return -1;
    }
    return steps;
}

extern "C" long shll_steps_for(const shll_params* p) {
    char e[128];
    if (shll_validate_params(p, e, sizeof(e)) != SHLL_OK) return -1;
    if (p->n_steps > 0) return p->n_steps;
    return clock_is_f32(p) ? count_steps_t<float>(p) : count_steps_t<double>(p);
}

// ---------------- initial conditions (host) ----------------
// Writes nv primitive planes (rho, u, [v,] T) in double.  The reference ICs:
// base-c/base_shll.c:53-60, base-c/base_shll_2d.c:92-103, base-c/2nd_order_base_shll.c:133-149.
void shll_ic_fill(const shll_params* p, int real_bits, double* prim) {
    const int nx = p->nx, ny = p->dim == 2 ? p->ny : 1;
    const size_t n = (size_t)nx * ny;
    const shll_ic& ic = p->ic;
    if (p->dim == 1) {
        for (int i = 0; i < nx; i++) {
            bool left = i < ic.x_d * nx;
            prim[i] = left ? ic.rho_l : ic.rho_r;
            prim[n + i] = left ? ic.u_l : ic.u_r;
            prim[2 * n + i] = left ? ic.T_l : ic.T_r;
        }
        return;
    }
    const double dx = p->lx / nx, dy = p->ly / ny;
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) {
            size_t c = (size_t)i * ny + j;
            double rho = 1, u = 0, v = 0, T = 1;
            if (ic.kind == SHLL_IC_REF_BOX2D) {
                bool in = (i > 0.2 * nx) && (i < 0.8 * nx) && (j > 0.2 * ny) && (j < 0.8 * ny);
                rho = in ? 1.0 : 10.0;
            } else if (ic.kind == SHLL_IC_CIRCLE2D) {
                double x = (i + 0.5) * dx - ic.cx, y = (j + 0.5) * dy - ic.cy;
                bool in = x * x + y * y < ic.radius * ic.radius;
                rho = in ? ic.rho_l : ic.rho_r;
                T = in ? ic.T_l : ic.T_r;
            } else if (ic.kind == SHLL_IC_QUADRANTS2D) {
                if ((i < 0.5 * nx) && (j < 0.5 * ny)) { rho = 1.0; u = -0.75; v = 0.5; }
                else if ((i > 0.5 * nx) && (j < 0.5 * ny)) { rho = 3.0; u = -0.75; v = -0.5; }
                else if ((i < 0.5 * nx) && (j > 0.5 * ny)) { rho = 2.0; u = 0.75; v = 0.5; }
                else { rho = 1.0; u = 0.75; v = -0.5; }
                T = real_bits == 32 ? (double)(float)(1.0 / (double)((float)rho * (float)p->R)) : 1.0 / (rho * p->R);
            } else if (ic.kind == SHLL_IC_FOUR_SHOCK2D) {
                double pr;
                if ((i < 0.75 * nx) && (j < 0.75 * ny)) { rho = 0.138; u = 1.206; v = 1.206; pr = 0.029; }
                else if ((i > 0.75 * nx) && (j < 0.75 * ny)) { rho = 0.5323; u = 0.0; v = 1.206; pr = 0.3; }
                else if ((i < 0.75 * nx) && (j > 0.75 * ny)) { rho = 0.5323; u = 1.206; v = 0.0; pr = 0.3; }
                else { rho = 1.5; u = 0.0; v = 0.0; pr = 1.5; }
                if (real_bits == 32) {  // p3 = pr/(p0*R) with p0*R in float, as the reference
                    float rf = (float)rho, Rf = (float)p->R;
                    rho = rf; u = (float)u; v = (float)v;
                    T = (float)(pr / (double)(rf * Rf));
                } else {
                    T = pr / (rho * p->R);
                }
            }
            prim[c] = rho; prim[n + c] = u; prim[2 * n + c] = v; prim[3 * n + c] = T;
        }
}

// ---------------- context ----------------
static PlainArgs plain_args(shll_ctx* c) {
    PlainArgs a;
    memset(&a, 0, sizeof(a));
    a.dim = c->p.dim; a.order = c->p.order; a.limiter = c->p.limiter; a.real_bits = c->real_bits;
    a.nx = c->p.nx; a.ny = c->p.dim == 2 ? c->p.ny : 1;
    a.Uin = c->U[c->cur]; a.Uout = c->U[c->cur];
    a.P = c->P; a.fp = c->F[0]; a.fm = c->F[1]; a.hp = c->F[2]; a.hm = c->F[3];
    a.R = c->R; a.GAMMA = c->GAMMA; a.CV = c->CV; a.DT_ON_DX = c->DT_ON_DX; a.DT_ON_DY = c->DT_ON_DY;
    a.mc_alpha = c->p.mc_alpha;
    a.flag = c->d_flag;
    a.stream = c->stream;
    return a;
}

static cudaError_t plain_step(shll_ctx* c, const PlainArgs& a) {
    return c->p.precision == SHLL_PREC_F64 ? plain_fast::step(a) : plain_exact::step(a);
}
static cudaError_t plain_stage(shll_ctx* c, const PlainArgs& a, int which) {
    return c->p.precision == SHLL_PREC_F64 ? plain_fast::stage(a, which) : plain_exact::stage(a, which);
}

extern "C" int shll_create(const shll_params* p, shll_ctx** out) {
    if (!out) return SHLL_ERR_ARG;
    *out = nullptr;
    char e[256];
    int rc = shll_validate_params(p, e, sizeof(e));
    if (rc != SHLL_OK) {
        fprintf(stderr, "shll_create: %s\n", e);
        return rc;
    }
    shll_ctx* c = new (std::nothrow) shll_ctx();
    if (!c) return SHLL_ERR_NOMEM;
    c->p = *p;
    if (c->p.dim == 1) c->p.ny = 1;
    c->nv = c->p.dim == 2 ? 4 : 3;
    c->n = c->p.nx * c->p.ny;
    c->plain = c->p.precision <= SHLL_PREC_F32_EXACT;
    c->real_bits = c->p.precision == SHLL_PREC_F32_EXACT ? 32 : 64;
    if (c->real_bits == 32)
        ref_constants<float>(&c->p, &c->R, &c->GAMMA, &c->CV, &c->DX, &c->DY, &c->DT, &c->DT_ON_DX, &c->DT_ON_DY);
    else
        ref_constants<double>(&c->p, &c->R, &c->GAMMA, &c->CV, &c->DX, &c->DY, &c->DT, &c->DT_ON_DX, &c->DT_ON_DY);
    c->steps_total = shll_steps_for(&c->p);
    cudaError_t ce = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (ce != cudaSuccess) {
        fprintf(stderr, "shll_create: cudaStreamCreate failed: %s\n", cudaGetErrorString(ce));
        delete c;
        return SHLL_ERR_CUDA;
    }
    c->own_stream = true;
    const size_t rb = c->real_bits / 8, n = (size_t)c->n;
    bool ok = cudaMalloc(&c->d_flag, sizeof(int)) == cudaSuccess;
    ok = ok && cudaMemset(c->d_flag, 0, sizeof(int)) == cudaSuccess;
    if (c->plain) {
        ok = ok && cudaMalloc(&c->U[0], c->nv * n * rb) == cudaSuccess;
        ok = ok && cudaMalloc(&c->U[1], c->nv * n * rb) == cudaSuccess;
        ok = ok && cudaMalloc(&c->P, (c->nv + 1) * n * rb) == cudaSuccess;
    } else {
        c->mixed = mixed_create(&c->p, c->DT_ON_DX, c->DT_ON_DY, c->CV, c->stream, c->err, sizeof(c->err));
        ok = ok && c->mixed != nullptr;
    }
    if (!ok) {
        fprintf(stderr, "shll_create: device allocation failed (%zu cells): %s\n", n, c->err);
        shll_destroy(c);
        return SHLL_ERR_NOMEM;
    }
    *out = c;
    return SHLL_OK;
}

extern "C" void shll_destroy(shll_ctx* c) {
    if (!c) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->U[0]); cudaFree(c->U[1]); cudaFree(c->P); cudaFree(c->ckU); cudaFree(c->ckP);
    for (int k = 0; k < 4; k++) cudaFree(c->F[k]);
    cudaFree(c->d_flag);
    if (c->mixed) mixed_destroy(c->mixed);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" const char* shll_last_error(const shll_ctx* c) { return c ? c->err : "no context"; }

extern "C" const char* shll_status_string(int s) {
    switch (s) {
        case SHLL_OK: return "ok";
        case SHLL_ERR_ARG: return "invalid argument";
        case SHLL_ERR_CUDA: return "CUDA error";
        case SHLL_ERR_STATE: return "call out of order";
        case SHLL_ERR_NOMEM: return "out of memory";
        case SHLL_ERR_NUMERIC: return "non-positive density or temperature";
        case SHLL_ERR_TIMEOUT: return "device wait timed out";
        case SHLL_ERR_UNSUPPORTED: return "unsupported for this configuration";
        default: return "unknown status";
    }
}

extern "C" int shll_set_stream(shll_ctx* c, void* s) {
    if (!c) return SHLL_ERR_ARG;
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    if (c->own_stream) cudaStreamDestroy(c->stream);
    c->own_stream = false;
    if (s) {
        c->stream = (cudaStream_t)s;
    } else {
        CUDA_TRY(c, cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
        c->own_stream = true;
    }
    if (c->mixed) mixed_set_stream(c->mixed, c->stream);
    return SHLL_OK;
}

// reads the error flag of the context's engine (the plain kernels' flag, or the mixed engine's)
static int check_flag(shll_ctx* c) {
    int h = 0;
    if (c->plain) {
        CUDA_TRY(c, cudaMemcpyAsync(&h, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    } else {
        h = mixed_flags(c->mixed);
        CUDA_TRY(c, cudaGetLastError());
    }
    if (h & SHLL_FLAG_TIMEOUT) { set_err(c, "a bounded device wait expired"); return SHLL_ERR_TIMEOUT; }
    if (h & SHLL_FLAG_BADARG) { set_err(c, "a kernel rejected its launch arguments"); return SHLL_ERR_ARG; }
    if (h & SHLL_FLAG_NONPOSITIVE) { set_err(c, "non-positive or NaN density/temperature reached"); return SHLL_ERR_NUMERIC; }
    return SHLL_OK;
}

// uploads double primitive planes, then U from P and P from U (base_shll.c:202-205)
// derive = false (plain paths only) leaves U to the caller's Compute_U_from_P, as the reference's
// Allocate_and_Init_Memory does
static int load_primitives(shll_ctx* c, const double* prim, bool derive = true) {
    const size_t n = (size_t)c->n, nv = c->nv;
    c->steps_taken = 0;
    c->fluxes_valid = false;
    CUDA_TRY(c, cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->stream));
    if (!c->plain) {
        int rc = mixed_load(c->mixed, prim, c->err, sizeof(c->err));
        if (rc != SHLL_OK) return rc;
        c->initialized = true;
        return check_flag(c);
    }
    std::vector<unsigned char> host(nv * n * (c->real_bits / 8));
    if (c->real_bits == 32) {
        float* h = reinterpret_cast<float*>(host.data());
        for (size_t i = 0; i < nv * n; i++) h[i] = (float)prim[i];
    } else {
        memcpy(host.data(), prim, nv * n * sizeof(double));
    }
    CUDA_TRY(c, cudaMemcpyAsync(c->P, host.data(), host.size(), cudaMemcpyHostToDevice, c->stream));
    c->cur = 0;
    if (derive) {
        PlainArgs a = plain_args(c);
        CUDA_TRY(c, plain_stage(c, a, STAGE_U_FROM_P));
        CUDA_TRY(c, plain_stage(c, a, STAGE_P_FROM_U));
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    c->initialized = true;
    return check_flag(c);
}

extern "C" int shll_init_state(shll_ctx* c) {
    if (!c) return SHLL_ERR_ARG;
    if (c->p.ic.kind == SHLL_IC_USER) {
        set_err(c, "initial condition is SHLL_IC_USER: call shll_set_primitives");
        return SHLL_ERR_STATE;
    }
    std::vector<double> prim((size_t)c->nv * c->n);
    shll_ic_fill(&c->p, c->real_bits, prim.data());
    return load_primitives(c, prim.data());
}

extern "C" int shll_initial_primitives(const shll_params* p, double* rho, double* u, double* v, double* T) {
    char e[256];
    if (!p || !rho || !u || !T || (p->dim == 2 && !v)) return SHLL_ERR_ARG;
    if (shll_validate_params(p, e, sizeof(e)) != SHLL_OK || p->ic.kind == SHLL_IC_USER) return SHLL_ERR_ARG;
    const size_t n = (size_t)p->nx * (p->dim == 2 ? p->ny : 1);
    const int nv = p->dim == 2 ? 4 : 3;
    std::vector<double> prim((size_t)nv * n);
    shll_ic_fill(p, p->precision == SHLL_PREC_F32_EXACT ? 32 : 64, prim.data());  // as shll_init_state
    double* out[4] = {rho, u, p->dim == 2 ? v : T, T};
    for (int k = 0; k < nv; k++) memcpy(out[k], prim.data() + (size_t)k * n, n * sizeof(double));
    return SHLL_OK;
}

extern "C" int shll_set_primitives(shll_ctx* c, const double* rho, const double* u, const double* v, const double* T) {
    if (!c || !rho || !u || !T || (c->p.dim == 2 && !v)) return SHLL_ERR_ARG;
    if (!c->plain) {  // copied as given and converted (and checked) on the device
        const double* planes[4] = {rho, u, c->p.dim == 2 ? v : T, T};
        c->steps_taken = 0;
        c->fluxes_valid = false;
        int rc = mixed_set_item_primitives(c->mixed, 0, planes, c->err, sizeof(c->err));
        if (rc != SHLL_OK) return rc;
        c->initialized = true;
        return check_flag(c);
    }
    const size_t n = (size_t)c->n;
    std::vector<double> prim(c->nv * n);
    memcpy(prim.data(), rho, n * sizeof(double));
    memcpy(prim.data() + n, u, n * sizeof(double));
    if (c->p.dim == 2) {
        memcpy(prim.data() + 2 * n, v, n * sizeof(double));
        memcpy(prim.data() + 3 * n, T, n * sizeof(double));
    } else {
        memcpy(prim.data() + 2 * n, T, n * sizeof(double));
    }
    for (size_t i = 0; i < n; i++) {
        double r = prim[i], t = prim[(c->nv - 1) * n + i];
        if (!(r > 0) || !(t > 0)) {
            set_err(c, "cell %zu: density and temperature must be positive", i);
            return SHLL_ERR_ARG;
        }
    }
    return load_primitives(c, prim.data());
}

static int stage_call(shll_ctx* c, int which) {
    if (!c) return SHLL_ERR_ARG;
    if (!c->initialized) { set_err(c, "state not initialised (call shll_init_state)"); return SHLL_ERR_STATE; }
    if (!c->plain) {
        set_err(c, "the reference's separate stages exist only for the F64/F32 precisions");
        return SHLL_ERR_UNSUPPORTED;
    }
    if (which == STAGE_F_FROM_P && !c->F[0]) {
        const size_t bytes = (size_t)c->nv * c->n * (c->real_bits / 8);
        for (int k = 0; k < (c->p.dim == 2 ? 4 : 2); k++) CUDA_TRY(c, cudaMalloc(&c->F[k], bytes));
    }
    if (which == STAGE_UPDATE && !c->fluxes_valid) {
        set_err(c, "Update_U_from_F before Compute_F_from_P");
        return SHLL_ERR_STATE;
    }
    PlainArgs a = plain_args(c);
    CUDA_TRY(c, plain_stage(c, a, which));
    if (which == STAGE_F_FROM_P) c->fluxes_valid = true;
    return SHLL_OK;
}

extern "C" int shll_compute_U_from_P(shll_ctx* c) { return stage_call(c, STAGE_U_FROM_P); }
extern "C" int shll_compute_P_from_U(shll_ctx* c) { return stage_call(c, STAGE_P_FROM_U); }
extern "C" int shll_compute_F_from_P(shll_ctx* c) { return stage_call(c, STAGE_F_FROM_P); }
extern "C" int shll_update_U_from_F(shll_ctx* c) { return stage_call(c, STAGE_UPDATE); }

extern "C" int shll_step(shll_ctx* c, long nsteps) {
    if (!c || nsteps < 0) return SHLL_ERR_ARG;
    if (!c->initialized) { set_err(c, "state not initialised (call shll_init_state)"); return SHLL_ERR_STATE; }
    if (nsteps == 0) return SHLL_OK;
    if (!c->plain) {
        int rc = mixed_step(c->mixed, nsteps, c->err, sizeof(c->err));
        if (rc != SHLL_OK) return rc;
        c->steps_taken += nsteps;
        return check_flag(c);
    }
    for (long s = 0; s < nsteps; s++) {
        PlainArgs a = plain_args(c);
        a.Uin = c->U[c->cur];
        a.Uout = c->U[c->cur ^ 1];
        CUDA_TRY(c, plain_step(c, a));
        c->cur ^= 1;
    }
    PlainArgs a = plain_args(c);
    CUDA_TRY(c, plain_stage(c, a, STAGE_P_FROM_U));  // the loop ends with Compute_P_from_U
    c->fluxes_valid = false;
    c->steps_taken += nsteps;
    return check_flag(c);
}

extern "C" int shll_run(shll_ctx* c, long* steps_taken) {
    if (!c) return SHLL_ERR_ARG;
    long remaining = c->steps_total - c->steps_taken;
    int rc = remaining > 0 ? shll_step(c, remaining) : SHLL_OK;
    if (steps_taken) *steps_taken = c->steps_taken;
    return rc;
}

extern "C" int shll_autotune(shll_ctx* c, int trial_steps) {
    if (!c) return SHLL_ERR_ARG;
    if (c->plain) { set_err(c, "the autotuner covers the mixed-precision engines"); return SHLL_ERR_UNSUPPORTED; }
    if (!c->initialized) { set_err(c, "state not initialised (call shll_init_state)"); return SHLL_ERR_STATE; }
    int rc = mixed_autotune(c->mixed, trial_steps, c->err, sizeof(c->err));
    if (rc == SHLL_OK) c->ck_steps = c->steps_taken;   // the device checkpoint now holds this state
    return rc;
}

extern "C" int shll_tuning(shll_ctx* c, int* sweep_steps, int* fold_steps, int* chunk_cells) {
    if (!c || c->plain) return SHLL_ERR_ARG;
    return mixed_tuning(c->mixed, 0, sweep_steps, fold_steps, chunk_cells);
}

extern "C" long shll_steps_taken(const shll_ctx* c) { return c ? c->steps_taken : -1; }

static std::atomic<long> g_launches{0};
void shll_count_launches(long n) { g_launches += n; }
extern "C" long shll_kernel_launches(void) { return g_launches.load(); }

extern "C" int shll_checkpoint(shll_ctx* c) {
    if (!c) return SHLL_ERR_ARG;
    if (!c->initialized) { set_err(c, "state not initialised"); return SHLL_ERR_STATE; }
    if (!c->plain) {
        int rc = mixed_checkpoint(c->mixed, false, c->err, sizeof(c->err));
        if (rc == SHLL_OK) c->ck_steps = c->steps_taken;
        return rc;
    }
    const size_t rb = c->real_bits / 8, n = (size_t)c->n;
    if (!c->ckU) {
        CUDA_TRY(c, cudaMalloc(&c->ckU, c->nv * n * rb));
        CUDA_TRY(c, cudaMalloc(&c->ckP, (c->nv + 1) * n * rb));
    }
    CUDA_TRY(c, cudaMemcpyAsync(c->ckU, c->U[c->cur], c->nv * n * rb, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->ckP, c->P, (c->nv + 1) * n * rb, cudaMemcpyDeviceToDevice, c->stream));
    c->ck_steps = c->steps_taken;
    c->ck_cur = c->cur;
    return SHLL_OK;
}

extern "C" int shll_restore(shll_ctx* c) {
    if (!c) return SHLL_ERR_ARG;
    if (c->ck_steps < 0) { set_err(c, "no checkpoint taken"); return SHLL_ERR_STATE; }
    if (!c->plain) {
        int rc = mixed_checkpoint(c->mixed, true, c->err, sizeof(c->err));
        if (rc == SHLL_OK) c->steps_taken = c->ck_steps;
        return rc;
    }
    const size_t rb = c->real_bits / 8, n = (size_t)c->n;
    c->cur = c->ck_cur;
    CUDA_TRY(c, cudaMemcpyAsync(c->U[c->cur], c->ckU, c->nv * n * rb, cudaMemcpyDeviceToDevice, c->stream));
    CUDA_TRY(c, cudaMemcpyAsync(c->P, c->ckP, (c->nv + 1) * n * rb, cudaMemcpyDeviceToDevice, c->stream));
    c->steps_taken = c->ck_steps;
    c->fluxes_valid = false;
    return SHLL_OK;
}

template <typename REAL>
static void widen(const std::vector<unsigned char>& src, size_t off, size_t n, double* dst) {
    const REAL* s = reinterpret_cast<const REAL*>(src.data()) + off;
    for (size_t i = 0; i < n; i++) dst[i] = (double)s[i];
}

// copies nplanes device planes (REAL) starting at plane0 of buffer dev into host doubles
static int fetch_planes(shll_ctx* c, const void* dev, int plane0, int nplanes, double** dst) {
    const size_t n = (size_t)c->n, rb = c->real_bits / 8;
    std::vector<unsigned char> h(nplanes * n * rb);
    CUDA_TRY(c, cudaMemcpyAsync(h.data(), static_cast<const unsigned char*>(dev) + plane0 * n * rb, h.size(),
                                cudaMemcpyDeviceToHost, c->stream));
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    for (int k = 0; k < nplanes; k++) {
        if (!dst[k]) continue;
        if (c->real_bits == 32) widen<float>(h, k * n, n, dst[k]);
        else widen<double>(h, k * n, n, dst[k]);
    }
    return SHLL_OK;
}

extern "C" int shll_get_primitives(shll_ctx* c, double* rho, double* u, double* v, double* T) {
    if (!c) return SHLL_ERR_ARG;
    if (!c->initialized) { set_err(c, "state not initialised"); return SHLL_ERR_STATE; }
    if (!c->plain) return mixed_get_primitives(c->mixed, rho, u, v, T, c->err, sizeof(c->err));
    double* d2[3] = {rho, u, T};
    double* d3[4] = {rho, u, v, T};
    return fetch_planes(c, c->P, 0, c->nv, c->p.dim == 2 ? d3 : d2);
}

extern "C" int shll_get_conserved(shll_ctx* c, double* planes) {
    if (!c || !planes) return SHLL_ERR_ARG;
    if (!c->initialized) { set_err(c, "state not initialised"); return SHLL_ERR_STATE; }
    if (!c->plain) return mixed_get_conserved(c->mixed, planes, c->err, sizeof(c->err));
    double* d[4];
    for (int k = 0; k < c->nv; k++) d[k] = planes + (size_t)k * c->n;
    return fetch_planes(c, c->U[c->cur], 0, c->nv, d);
}

extern "C" int shll_get_fluxes(shll_ctx* c, double* fp, double* fm, double* hp, double* hm) {
    if (!c || !fp || !fm) return SHLL_ERR_ARG;
    if (!c->fluxes_valid) { set_err(c, "no split fluxes: call shll_compute_F_from_P"); return SHLL_ERR_STATE; }
    double* q[4] = {fp, fm, hp, hm};
    for (int f = 0; f < (c->p.dim == 2 ? 4 : 2); f++) {
        if (!q[f]) continue;
        double* d[4];
        for (int k = 0; k < c->nv; k++) d[k] = q[f] + (size_t)k * c->n;
        int rc = fetch_planes(c, c->F[f], 0, c->nv, d);
        if (rc != SHLL_OK) return rc;
    }
    return SHLL_OK;
}

extern "C" int shll_totals(shll_ctx* c, double* out) {
    if (!c || !out) return SHLL_ERR_ARG;
    if (!c->initialized) { set_err(c, "state not initialised"); return SHLL_ERR_STATE; }
    if (!c->plain) return mixed_totals(c->mixed, out, c->err, sizeof(c->err));
    cudaError_t e = device_plane_sums(c->U[c->cur], c->real_bits, c->nv, c->n, out, c->stream);
    if (e != cudaSuccess) { set_err(c, "totals: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    return SHLL_OK;
}

// Save_Results: base_shll.c:180-192 (1D), base_shll_2d.c:322-340 (2D); cell centres are
// computed in the reference's float: cx = (i+0.5)*DX with float DX.
extern "C" int shll_save_results(shll_ctx* c, const char* path) {
    if (!c || !path) return SHLL_ERR_ARG;
    const size_t n = (size_t)c->n;
    std::vector<double> pr(c->nv * n);
    int rc = c->p.dim == 2 ? shll_get_primitives(c, pr.data(), pr.data() + n, pr.data() + 2 * n, pr.data() + 3 * n)
                           : shll_get_primitives(c, pr.data(), pr.data() + n, nullptr, pr.data() + 2 * n);
    if (rc != SHLL_OK) return rc;
    FILE* f = fopen(path, "w");
    if (!f) { set_err(c, "cannot open %s for writing", path); return SHLL_ERR_ARG; }
    float DX = (float)c->p.lx / (float)c->p.nx, DY = (float)c->p.ly / (float)(c->p.dim == 2 ? c->p.ny : 1);
    if (c->p.dim == 1) {
        for (int i = 0; i < c->p.nx; i++) {
            float cx = (float)((i + 0.5) * DX);
            fprintf(f, "%e\t%e\t%e\t%e\n", cx, pr[i], pr[n + i], pr[2 * n + i]);
        }
    } else {
        size_t idx = 0;
        for (int i = 0; i < c->p.nx; i++)
            for (int j = 0; j < c->p.ny; j++, idx++) {
                float cx = (float)((i + 0.5) * DX), cy = (float)((j + 0.5) * DY);
                fprintf(f, "%e\t%e\t%e\t%e\t%e\t%e\n", cx, cy, pr[idx], pr[n + idx], pr[2 * n + idx], pr[3 * n + idx]);
            }
    }
    fclose(f);
    return SHLL_OK;
}

// ---------------- the reference's entry points on a default context ----------------
static shll_params g_ref_params;
static bool g_ref_configured = false;
static bool g_ref_program = false;   // configured from the loading program's reference globals
static shll_ctx* g_ref = nullptr;

extern "C" int shll_ref_configure(const shll_params* p) {
    char e[256];
    int rc = shll_validate_params(p, e, sizeof(e));
    if (rc != SHLL_OK) { fprintf(stderr, "shll_ref_configure: %s\n", e); return rc; }
    g_ref_params = *p;
    g_ref_configured = true;
    return SHLL_OK;
}

extern "C" shll_ctx* shll_ref_context(void) { return g_ref; }

static void ref_fail(const char* what, int rc) {
    fprintf(stderr, "%s: %s (%s)\n", what, shll_status_string(rc), g_ref ? g_ref->err : "");
}

extern "C" void Allocate_and_Init_Memory(void) {
    if (!g_ref_configured) {
        // a reference program linked against the library: its own problem; else base_shll.c's defaults
        g_ref_program = shll_ref_program_params(&g_ref_params);
        if (!g_ref_program) shll_params_default(&g_ref_params, 1, 1);
        g_ref_configured = true;
    }
    if (g_ref) { shll_destroy(g_ref); g_ref = nullptr; }
    int rc = shll_create(&g_ref_params, &g_ref);
    if (rc != SHLL_OK) { ref_fail("Allocate_and_Init_Memory", rc); return; }
    // The reference only sets P here; its main then calls Compute_U_from_P and Compute_P_from_U
    // (base_shll.c:202-205).  The plain paths load P alone so that those calls are the first and
    // only ones (in FP32 the U -> P -> U round trip is not idempotent); the mixed engine, which
    // has no separate stages, initialises its state completely.
    if (g_ref_params.ic.kind == SHLL_IC_USER) {
        ref_fail("Allocate_and_Init_Memory", SHLL_ERR_STATE);
        return;
    }
    std::vector<double> prim((size_t)g_ref->nv * g_ref->n);
    shll_ic_fill(&g_ref->p, g_ref->real_bits, prim.data());
    rc = load_primitives(g_ref, prim.data(), !g_ref->plain);
    if (rc != SHLL_OK) ref_fail("Allocate_and_Init_Memory", rc);
}
#define REF_STAGE(NAME, CALL)                                      \
    extern "C" void NAME(void) {                                   \
        if (!g_ref) { fprintf(stderr, #NAME ": no state\n"); return; } \
        int rc = CALL(g_ref);                                      \
        if (rc != SHLL_OK) ref_fail(#NAME, rc);                    \
    }
extern "C" void Compute_U_from_P(void) {
    if (!g_ref) { fprintf(stderr, "Compute_U_from_P: no state\n"); return; }
    int rc = shll_compute_U_from_P(g_ref);
    if (rc != SHLL_OK) ref_fail("Compute_U_from_P", rc);
    // and, as the reference's, the step globals that its main() reads
    if (g_ref_program) shll_ref_set_step(g_ref->DT, g_ref->DT_ON_DX, g_ref->DT_ON_DY);
}
REF_STAGE(Compute_P_from_U, shll_compute_P_from_U)
REF_STAGE(Compute_F_from_P, shll_compute_F_from_P)
REF_STAGE(Update_U_from_F, shll_update_U_from_F)

extern "C" void Save_Results(void) {
    if (!g_ref) { fprintf(stderr, "Save_Results: no state\n"); return; }
    int rc = shll_save_results(g_ref, "results.dat");
    if (rc != SHLL_OK) ref_fail("Save_Results", rc);
}

extern "C" void Free_Memory(void) {
    shll_destroy(g_ref);
    g_ref = nullptr;
}

extern "C" double shll_ref_dt(void) { return g_ref ? g_ref->DT : 0.0; }

// ---------------- batches ----------------
struct shll_batch {
    MixedState* m = nullptr;     // mixed-precision items
    PlainBatch* pb = nullptr;    // SHLL_PREC_F64 / F64_EXACT items (one launch per step)
    cudaStream_t stream = nullptr;
    int count = 0;
    bool loaded = false;
    char err[512] = {0};
};

extern "C" int shll_batch_create(const shll_params* items, int count, shll_batch** out) {
    if (!out || !items || count <= 0) return SHLL_ERR_ARG;
    *out = nullptr;
    char e[256];
    for (int i = 0; i < count; i++) {
        int rc = shll_validate_params(&items[i], e, sizeof(e));
        if (rc != SHLL_OK) { fprintf(stderr, "shll_batch_create: item %d: %s\n", i, e); return rc; }
        if (items[i].ic.kind == SHLL_IC_USER) {
            fprintf(stderr, "shll_batch_create: item %d: batches take descriptor initial conditions\n", i);
            return SHLL_ERR_ARG;
        }
    }
    const int prec = items[0].precision;
    for (int i = 1; i < count; i++)
        if (items[i].precision != prec || items[i].dim != items[0].dim) {
            fprintf(stderr, "shll_batch_create: item %d: batch items share one dimension and one precision\n", i);
            return SHLL_ERR_ARG;
        }
    if (prec == SHLL_PREC_F32_EXACT) {
        fprintf(stderr, "shll_batch_create: batches take F64, F64_EXACT or the mixed precisions\n");
        return SHLL_ERR_UNSUPPORTED;
    }
    shll_batch* b = new (std::nothrow) shll_batch();
    if (!b) return SHLL_ERR_NOMEM;
    b->count = count;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) { delete b; return SHLL_ERR_CUDA; }
    int rc;
    if (prec == SHLL_PREC_F64 || prec == SHLL_PREC_F64_EXACT) {
        b->pb = plain_batch_create(items, count, b->stream, b->err, sizeof(b->err));
        if (!b->pb) {
            fprintf(stderr, "shll_batch_create: %s\n", b->err);
            cudaStreamDestroy(b->stream);
            delete b;
            return SHLL_ERR_ARG;
        }
        rc = plain_batch_load(b->pb, b->err, sizeof(b->err));
    } else {
        b->m = mixed_create_batch(items, count, b->stream, b->err, sizeof(b->err));
        if (!b->m) {
            fprintf(stderr, "shll_batch_create: %s\n", b->err);
            cudaStreamDestroy(b->stream);
            delete b;
            return SHLL_ERR_NOMEM;
        }
        rc = mixed_load_all(b->m, b->err, sizeof(b->err));
    }
    if (rc != SHLL_OK) { shll_batch_destroy(b); return rc; }
    b->loaded = true;
    *out = b;
    return SHLL_OK;
}

extern "C" int shll_batch_run(shll_batch* b) {
    if (!b) return SHLL_ERR_ARG;
    int rc = b->pb ? plain_batch_run(b->pb, b->err, sizeof(b->err)) : mixed_step(b->m, -1, b->err, sizeof(b->err));
    if (rc != SHLL_OK) return rc;
    int f = b->pb ? plain_batch_flags(b->pb) : mixed_flags(b->m);
    if (f & SHLL_FLAG_TIMEOUT) { snprintf(b->err, sizeof(b->err), "a bounded device wait expired"); return SHLL_ERR_TIMEOUT; }
    if (f & SHLL_FLAG_BADARG) { snprintf(b->err, sizeof(b->err), "a kernel rejected its launch arguments"); return SHLL_ERR_ARG; }
    if (f & SHLL_FLAG_NONPOSITIVE) { snprintf(b->err, sizeof(b->err), "non-positive density/energy reached"); return SHLL_ERR_NUMERIC; }
    return SHLL_OK;
}

extern "C" int shll_batch_set_stream(shll_batch* b, void* stream) {
    if (!b) return SHLL_ERR_ARG;
    cudaStream_t s = stream ? (cudaStream_t)stream : b->stream;
    if (b->m) mixed_set_stream(b->m, s);
    if (b->pb) plain_batch_set_stream(b->pb, s);
    return SHLL_OK;
}

extern "C" int shll_batch_get_primitives(shll_batch* b, int item, double* rho, double* u, double* v, double* T) {
    if (!b) return SHLL_ERR_ARG;
    if (b->pb) return plain_batch_item_primitives(b->pb, item, rho, u, v, T, b->err, sizeof(b->err));
    return mixed_item_primitives(b->m, item, rho, u, v, T, b->err, sizeof(b->err));
}

extern "C" int shll_batch_set_primitives(shll_batch* b, int item, const double* rho, const double* u, const double* v,
                                         const double* T) {
    if (!b || item < 0 || item >= b->count || !rho || !u || !T) return SHLL_ERR_ARG;
    if (!b->m) {
        snprintf(b->err, sizeof(b->err), "host primitives for batch items need a mixed-precision batch");
        return SHLL_ERR_UNSUPPORTED;
    }
    int count = 0;
    const shll_params* items = mixed_items(b->m, &count);
    const bool two_d = items[item].dim == 2;
    if (two_d && !v) return SHLL_ERR_ARG;
    const double* planes[4] = {rho, u, two_d ? v : T, T};
    return mixed_set_item_primitives(b->m, item, planes, b->err, sizeof(b->err));
}

extern "C" int shll_batch_set_all_primitives(shll_batch* b, const double* prim) {
    if (!b || !prim) return SHLL_ERR_ARG;
    if (!b->m) {
        snprintf(b->err, sizeof(b->err), "host primitives for batch items need a mixed-precision batch");
        return SHLL_ERR_UNSUPPORTED;
    }
    return mixed_set_all_primitives(b->m, prim, b->err, sizeof(b->err));
}

extern "C" int shll_batch_get_all_primitives(shll_batch* b, double* prim) {
    if (!b || !prim) return SHLL_ERR_ARG;
    if (!b->m) {
        snprintf(b->err, sizeof(b->err), "packed primitives need a mixed-precision batch");
        return SHLL_ERR_UNSUPPORTED;
    }
    return mixed_get_all_primitives(b->m, prim, b->err, sizeof(b->err));
}

extern "C" int shll_batch_totals(shll_batch* b, int item, double* out) {
    if (!b || !out) return SHLL_ERR_ARG;
    if (b->pb) return plain_batch_item_totals(b->pb, item, out, b->err, sizeof(b->err));
    return mixed_item_totals(b->m, item, out, b->err, sizeof(b->err));
}

extern "C" int shll_batch_item_status(shll_batch* b, int item) {
    if (!b || item < 0 || item >= b->count) return SHLL_ERR_ARG;
    const int f = b->pb ? plain_batch_item_flags(b->pb, item) : mixed_item_flags(b->m, item);
    return (f & SHLL_FLAG_NONPOSITIVE) ? SHLL_ERR_NUMERIC : SHLL_OK;
}

extern "C" long shll_batch_cell_updates(const shll_batch* b) {
    if (!b) return -1;
    return b->pb ? plain_batch_cell_updates(b->pb) : mixed_cell_updates(b->m);
}
extern "C" const char* shll_batch_last_error(const shll_batch* b) { return b ? b->err : "no batch"; }

// autotuner of the mixed 1D engine (state restored afterwards) and its choices per item
extern "C" int shll_batch_autotune(shll_batch* b, int trial_steps) {
    if (!b) return SHLL_ERR_ARG;
    if (!b->m) { snprintf(b->err, sizeof(b->err), "the autotuner needs a mixed-precision batch"); return SHLL_ERR_UNSUPPORTED; }
    return mixed_autotune(b->m, trial_steps, b->err, sizeof(b->err));
}

extern "C" int shll_batch_tuning(shll_batch* b, int item, int* sweep_steps, int* fold_steps, int* chunk_cells) {
    if (!b || !b->m || item < 0 || item >= b->count) return SHLL_ERR_ARG;
    return mixed_tuning(b->m, item, sweep_steps, fold_steps, chunk_cells);
}

// device-side checkpoint / restore of a mixed-precision 1D batch (restore also clears the
// breakdown flags raised after the checkpoint)
extern "C" int shll_batch_checkpoint(shll_batch* b) {
    if (!b) return SHLL_ERR_ARG;
    if (!b->m) { snprintf(b->err, sizeof(b->err), "checkpoint needs a mixed-precision batch"); return SHLL_ERR_UNSUPPORTED; }
    if (!b->loaded) { snprintf(b->err, sizeof(b->err), "batch not loaded"); return SHLL_ERR_STATE; }
    return mixed_checkpoint(b->m, false, b->err, sizeof(b->err));
}

extern "C" int shll_batch_restore(shll_batch* b) {
    if (!b) return SHLL_ERR_ARG;
    if (!b->m) { snprintf(b->err, sizeof(b->err), "restore needs a mixed-precision batch"); return SHLL_ERR_UNSUPPORTED; }
    return mixed_checkpoint(b->m, true, b->err, sizeof(b->err));
}

extern "C" void shll_batch_destroy(shll_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->m) mixed_destroy(b->m);
    if (b->pb) plain_batch_destroy(b->pb);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
}

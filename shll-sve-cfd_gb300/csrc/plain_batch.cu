// Plain FP64 batches (SHLL_PREC_F64 or SHLL_PREC_F64_EXACT items of shll_batch_*): many
// independent tubes or domains, one launch per time step (per order) over the blocks of every
// item that still has steps.  The per-block arithmetic is the plain single-problem kernel's
// (shll_plain.cuh): the reference's FP64 arithmetic with fused multiply-add allowed (the kernels
// of this unit), or without it, bit-identical to the FP64 reference build (plain_batch_exact.cu).
#define SHLL_PLAIN_NS plain_batch_ns
#include "plain_batch_kernels.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "plain_batch.h"



using namespace plain_batch_ns;

// the kernels of plain_batch_exact.cu (the same item and block layouts, from the same header)
cudaError_t plain_batch_exact_launch(int dim, int order, int nb, cudaStream_t s, const void* items, const void* blks,
                                     double* U0, double* U1, long plane, int step, int* flags);

struct PlainBatch {
    int dim = 1, count = 0, nv = 3;
    bool exact = false;        // SHLL_PREC_F64_EXACT items
    cudaStream_t stream = nullptr;
    std::vector<shll_params> params;
    std::vector<PItem> items;
    std::vector<PBlk> blk[2];  // by order
    std::vector<int> par;
    long plane = 0, cell_updates = 0;
    double* U[2] = {nullptr, nullptr};
    PItem* d_items = nullptr;
    PBlk* d_blk[2] = {nullptr, nullptr};
    int* d_flag = nullptr;
};

PlainBatch* plain_batch_create(const shll_params* p, int count, cudaStream_t s, char* err, size_t len) {
    PlainBatch* b = new PlainBatch();
    b->stream = s;
    b->count = count;
    b->dim = p[0].dim;
    b->nv = b->dim == 2 ? 4 : 3;
    b->params.assign(p, p + count);
    b->exact = p[0].precision == SHLL_PREC_F64_EXACT;
    long off = 0;
    for (int t = 0; t < count; t++) {
        const shll_params& q = p[t];
        if (q.dim != b->dim || q.precision != p[0].precision ||
            (q.precision != SHLL_PREC_F64 && q.precision != SHLL_PREC_F64_EXACT)) {
            snprintf(err, len, "plain batches take SHLL_PREC_F64 or SHLL_PREC_F64_EXACT items of one dimension and "
                               "one precision");
            delete b;
            return nullptr;
        }
        PItem it;
        memset(&it, 0, sizeof(it));
        it.base = off;
        it.nx = q.nx;
        it.ny = b->dim == 2 ? q.ny : 1;
        it.order = q.order;
        // the reference's FP64 constants (base_shll.c:17-26, :83-84; base_shll_2d.c:134-136)
        const double R = q.R, G = q.gamma;
        const double CV = R / (G - 1.0), dx = q.lx / q.nx, dy = q.ly / it.ny;
        const double dt = (q.cfl / (R + 1)) * dx;
        it.g.R = R; it.g.GAMMA = G; it.g.CV = CV;
        it.g.DT_ON_DX = q.cfl / (R + 1);
        it.g.DT_ON_DY = dt / dy;
        it.g.alpha = q.mc_alpha;
        it.g.limiter = q.limiter;
        b->items.push_back(it);
        off += (long)it.nx * it.ny;
    }
    b->plane = off;
    b->par.assign(count, 0);
    bool ok = true;
    for (int k = 0; k < 2 && ok; k++) ok = cudaMalloc(&b->U[k], sizeof(double) * b->nv * off) == cudaSuccess;
    if (ok) ok = cudaMalloc(&b->d_items, sizeof(PItem) * count) == cudaSuccess;
    if (ok) ok = cudaMalloc(&b->d_flag, sizeof(int) * count) == cudaSuccess &&
                 cudaMemset(b->d_flag, 0, sizeof(int) * count) == cudaSuccess;  // one flag per item
    if (!ok) {
        snprintf(err, len, "plain batch: device allocation failed (%ld cells)", off);
        plain_batch_destroy(b);
        return nullptr;
    }
    return b;
}

void plain_batch_destroy(PlainBatch* b) {
    if (!b) return;
    for (int k = 0; k < 2; k++) { cudaFree(b->U[k]); cudaFree(b->d_blk[k]); }
    cudaFree(b->d_items);
    cudaFree(b->d_flag);
    delete b;
}

void plain_batch_set_stream(PlainBatch* b, cudaStream_t s) { b->stream = s; }

// U from P in FP64 (base_shll.c:76-80, base_shll_2d.c:126-131), for every item
int plain_batch_load(PlainBatch* b, char* err, size_t len) {
    std::vector<double> h((size_t)b->nv * b->plane);
    for (int t = 0; t < b->count; t++) {
        const shll_params& q = b->params[t];
        const PItem& it = b->items[t];
        const size_t n = (size_t)it.nx * it.ny;
        std::vector<double> prim(b->nv * n);
        shll_ic_fill(&q, 64, prim.data());
        const double CV = it.g.CV;
        for (size_t c = 0; c < n; c++) {
            const double p0 = prim[c], p1 = prim[n + c];
            double* U = h.data() + it.base + c;
            U[0] = p0;
            U[b->plane] = p0 * p1;
            if (b->nv == 3) {
                const double p2 = prim[2 * n + c];
                U[2 * b->plane] = p0 * (p2 * CV + 0.5 * p1 * p1);
            } else {
                const double p2 = prim[2 * n + c], p3 = prim[3 * n + c];
                U[2 * b->plane] = p0 * p2;
                U[3 * b->plane] = p0 * (p3 * CV + 0.5 * (p1 * p1 + p2 * p2));
            }
        }
        b->par[t] = 0;
    }
    if (cudaMemcpyAsync(b->U[0], h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess) {
        snprintf(err, len, "plain batch upload failed");
        return SHLL_ERR_CUDA;
    }
    return SHLL_OK;
}

int plain_batch_run(PlainBatch* b, char* err, size_t len) {
    long maxsteps = 0;
    for (int t = 0; t < b->count; t++) {
        b->items[t].steps = (int)shll_steps_for(&b->params[t]);
        b->items[t].par = b->par[t];
        maxsteps = std::max<long>(maxsteps, b->items[t].steps);
    }
    // blocks of each order, ordered by their item's steps, so step k covers a prefix
    for (int o = 0; o < 2; o++) b->blk[o].clear();
    for (int t = 0; t < b->count; t++) {
        const PItem& it = b->items[t];
        std::vector<PBlk>& v = b->blk[it.order - 1];
        if (b->dim == 1) {
            for (int a = 0; a < it.nx; a += T1) v.push_back({t, a, 0});
        } else {
            for (int a = 0; a < it.nx; a += TI)
                for (int c = 0; c < it.ny; c += TJ) v.push_back({t, a, c});
        }
    }
    std::vector<std::vector<int>> active(2, std::vector<int>(maxsteps + 2, 0));
    for (int o = 0; o < 2; o++) {
        std::stable_sort(b->blk[o].begin(), b->blk[o].end(),
                         [&](const PBlk& x, const PBlk& y) { return b->items[x.item].steps > b->items[y.item].steps; });
        // active[s] = blocks whose item has at least s steps (suffix sum of a histogram); step s
        // (0-based) runs the active[s + 1] blocks whose item has more than s steps
        for (const PBlk& k : b->blk[o]) active[o][b->items[k.item].steps]++;
        for (long s = maxsteps - 1; s >= 0; s--) active[o][s] += active[o][s + 1];
        cudaFree(b->d_blk[o]);
        b->d_blk[o] = nullptr;
        if (!b->blk[o].empty() &&
            (cudaMalloc(&b->d_blk[o], sizeof(PBlk) * b->blk[o].size()) != cudaSuccess ||
             cudaMemcpyAsync(b->d_blk[o], b->blk[o].data(), sizeof(PBlk) * b->blk[o].size(), cudaMemcpyHostToDevice,
                             b->stream) != cudaSuccess)) {
            snprintf(err, len, "plain batch: block list upload failed");
            return SHLL_ERR_CUDA;
        }
    }
    if (cudaMemcpyAsync(b->d_items, b->items.data(), sizeof(PItem) * b->count, cudaMemcpyHostToDevice, b->stream) != cudaSuccess) {
        snprintf(err, len, "plain batch: item upload failed");
        return SHLL_ERR_CUDA;
    }
    long launches = 0;
    cudaError_t e = cudaSuccess;
    for (long s = 0; s < maxsteps && e == cudaSuccess; s++) {
        for (int o = 0; o < 2 && e == cudaSuccess; o++) {
            const int nb = active[o][s + 1];
            if (nb == 0) continue;
            launches++;
            e = b->exact ? plain_batch_exact_launch(b->dim, o + 1, nb, b->stream, b->d_items, b->d_blk[o], b->U[0],
                                                    b->U[1], b->plane, (int)s, b->d_flag)
                         : batch_launch(b->dim, o + 1, nb, b->stream, b->d_items, b->d_blk[o], b->U[0], b->U[1],
                                        b->plane, (int)s, b->d_flag);
        }
    }
    shll_count_launches(launches);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) { snprintf(err, len, "plain batch launch failed: %s", cudaGetErrorString(e)); return SHLL_ERR_CUDA; }
    for (int t = 0; t < b->count; t++) {
        b->par[t] = (b->par[t] + b->items[t].steps) & 1;
        b->cell_updates += (long)b->items[t].steps * b->items[t].nx * b->items[t].ny;
    }
    return SHLL_OK;
}

int plain_batch_flags(PlainBatch* b) {
    std::vector<int> h(b->count);
    cudaMemcpyAsync(h.data(), b->d_flag, sizeof(int) * b->count, cudaMemcpyDeviceToHost, b->stream);
    cudaStreamSynchronize(b->stream);
    int f = 0;
    for (int v : h) f |= v;
    return f;
}

int plain_batch_item_flags(PlainBatch* b, int t) {
    if (t < 0 || t >= b->count) return 0;
    int h = 0;
    cudaMemcpyAsync(&h, b->d_flag + t, sizeof(int), cudaMemcpyDeviceToHost, b->stream);
    cudaStreamSynchronize(b->stream);
    return h;
}

long plain_batch_cell_updates(const PlainBatch* b) { return b->cell_updates; }

int plain_batch_item_primitives(PlainBatch* b, int t, double* rho, double* u, double* v, double* T, char* err,
                                size_t len) {
    if (t < 0 || t >= b->count) { snprintf(err, len, "item %d out of range", t); return SHLL_ERR_ARG; }
    const PItem& it = b->items[t];
    const size_t n = (size_t)it.nx * it.ny;
    std::vector<double> U(b->nv * n);
    for (int k = 0; k < b->nv; k++) {
        if (cudaMemcpyAsync(U.data() + k * n, b->U[b->par[t]] + k * b->plane + it.base, sizeof(double) * n,
                            cudaMemcpyDeviceToHost, b->stream) != cudaSuccess) {
            snprintf(err, len, "plain batch download failed");
            return SHLL_ERR_CUDA;
        }
    }
    if (cudaStreamSynchronize(b->stream) != cudaSuccess) { snprintf(err, len, "plain batch download failed"); return SHLL_ERR_CUDA; }
    const double CV = it.g.CV;
    for (size_t c = 0; c < n; c++) {
        const double u0 = U[c], p1 = U[n + c] / u0;
        if (rho) rho[c] = u0;
        if (u) u[c] = p1;
        if (b->nv == 3) {
            if (T) T[c] = ((U[2 * n + c] / u0) - 0.5 * p1 * p1) / CV;
        } else {
            const double p2 = U[2 * n + c] / u0;
            if (v) v[c] = p2;
            if (T) T[c] = ((U[3 * n + c] / u0) - 0.5 * (p1 * p1 + p2 * p2)) / CV;
        }
    }
    return SHLL_OK;
}

int plain_batch_item_totals(PlainBatch* b, int t, double* out, char* err, size_t len) {
    if (t < 0 || t >= b->count) { snprintf(err, len, "item %d out of range", t); return SHLL_ERR_ARG; }
    const PItem& it = b->items[t];
    for (int k = 0; k < b->nv; k++) {
        cudaError_t e = device_plane_sums(b->U[b->par[t]] + k * b->plane + it.base, 64, 1, (long)it.nx * it.ny, &out[k], b->stream);
        if (e != cudaSuccess) { snprintf(err, len, "plain batch totals failed"); return SHLL_ERR_CUDA; }
    }
    return SHLL_OK;
}

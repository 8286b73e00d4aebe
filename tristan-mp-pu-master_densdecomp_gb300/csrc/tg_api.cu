// C-ABI of the GB300 TRISTAN-MP hot path: context, device memory, the
// per-subroutine entry points and the fused, graph-captured lap.
#include <cuda_runtime.h>
#include <sys/mman.h>
#include <unistd.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <nvtx3/nvToolsExt.h>

#include "tg_internal.cuh"
#include "tg_spectrum.cuh"

using namespace tg;

// An NVTX range over one host entry point, named after the reference
// subroutine it replaces, so a timeline (nsys, ncu --nvtx) shows the main
// loop's phases; costs nothing when no tool is attached.
namespace {
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
}  // namespace
#define TG_RANGE(name) NvtxRange tg_nvtx_range_(name)

static thread_local char g_init_error[512];

// phase timers: TG_NPHASES of tristan_gpu.h

struct tg_ctx {
    tg_config cfg;
    Geom g;
    Params P;
    cudaStream_t st = nullptr;
    int device = 0;
    // device fields: ex ey ez bx by bz curx cury curz
    float *f[9] = {};
    float *ftmp[3] = {};   // filter ping-pong
    float4 *prim = nullptr;  // 3D primal copies, two float4 per cell (interleaved)
    unsigned long long *fix[3] = {};
    // particles: [parity][species]
    Species sp[2][2];
    int par = 0;
    long long *d_cnt = nullptr;  // [parity][species]
    long long hcount[2] = {0, 0};
    int *tstart[2] = {}, *hist[2] = {}, *cursor[2] = {};
    int *d_status = nullptr;
    int *d_dead = nullptr;  // a particle was dropped on purpose since the last sort
    bool fault_seen = false;  // a reported device fault may have dropped particles
    bool dirty = true;      // particles not grouped by tile
    bool may_have_dead = false;  // entries marked discarded since the last sort
    // host bindings
    float *hf[9] = {};
    void *hp = nullptr;
    int32_t *hions = nullptr, *hlecs = nullptr;
    // staging / scratch
    void *stage = nullptr;
    int *rk[4] = {};        // reorder keys in/out, values in/out
    void *cub_tmp = nullptr;
    size_t cub_bytes = 0;
    // FP64 diagnostics
    unsigned long long *rhofx = nullptr;
    double *rho[2] = {};
    double *dacc = nullptr, *dhist = nullptr;
    unsigned long long *dcounter = nullptr;
    int hist_cap = 1024;
    // graphs: one cycle of 2*sort_every laps per starting parity
    cudaGraphExec_t cycle[2] = {nullptr, nullptr};
    int kernels_per_step = 0;
    // phase timing: events per lap of a cycle, [lap][phase][begin/end]
    bool timing = false;
    std::vector<cudaEvent_t> ev;
    int ev_laps = 0;
    int last_laps = 0;       // laps covered by the last launch (graph or direct)
    bool last_direct = false;  // last lap ran outside the graph (event row ev_laps)
    bool ev_used[65][TG_NPHASES] = {};
    long long lap = 0;
    long long lapreorder = 0;
    // collisionless-shock hooks
    bool shock_on = false;
    ShockParams K;
    ShockState *d_shock = nullptr;
    float *d_tables = nullptr;  // gt_i, pt_i, gt_e, pt_e
    tg_shock hshock;
    // grid-moment scratch (FP64 sums)
    double *mom[2] = {};
    // host-driven laps (tg_step_host): copy streams, events (one link, then
    // uploaded / pushed per species and part), staging copy of the host
    // records (both species), the parts each species travels in
    cudaStream_t st_up = nullptr, st_down = nullptr;
    cudaEvent_t ev_link[1 + 4 * TG_HOST_PARTS_MAX] = {};
    void *stage2 = nullptr;
    long long host_n[2] = {0, 0};
    int host_parts = 0;                        // 0: by size
    int *ptstart[2][TG_HOST_PARTS_MAX] = {};   // tile starts of parts 1.. (part 0: tstart)
    long long *d_pcnt = nullptr;               // [species][part][records, sorted]
    long long pcnt[2][TG_HOST_PARTS_MAX][2] = {};
    std::vector<void *> pinned;  // host ranges page-locked by tg_pin_host
    char err[512] = {0};
    std::vector<void *> allocs;
};

static int fail(tg_ctx *c, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) snprintf(c->err, sizeof c->err, "%s", buf);
    else snprintf(g_init_error, sizeof g_init_error, "%s", buf);
    return code;
}

#define CK(call)                                                                                 \
    do {                                                                                         \
        cudaError_t e__ = (call);                                                                \
        if (e__ != cudaSuccess)                                                                  \
            return fail(ctx, TG_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e__), \
                        __FILE__, __LINE__);                                                     \
    } while (0)

template <class T>
static int dalloc(tg_ctx *ctx, T **p, size_t n) {
    void *q = nullptr;
    CK(cudaMalloc(&q, n * sizeof(T) + 256));
    ctx->allocs.push_back(q);
    *p = (T *)q;
    return TG_OK;
}

static int check_status(tg_ctx *ctx) {
    int st = 0;
    CK(cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    if (st == 0) return TG_OK;
    ctx->fault_seen = true;
    CK(cudaMemsetAsync(ctx->d_status, 0, sizeof(int), ctx->st));
    if (st & ST_NAN) return fail(ctx, TG_ERR_NAN, "non-finite particle coordinate (device status %d)", st);
    if (st & ST_OVERFLOW) return fail(ctx, TG_ERR_OVERFLOW, "particle capacity exceeded (device status %d)", st);
    if (st & ST_CHARGE_GRID)
        return fail(ctx, TG_ERR_OVERFLOW, "diagnostics: a node holds 2^17 particle charges or more (device status %d)", st);
    return fail(ctx, TG_ERR_BOUNDS, "particle or deposit outside the local grid (device status %d)", st);
}

// ---------------------------------------------------------------------------
// geometry
// ---------------------------------------------------------------------------
// failures write their message to err[0..errlen)
static int geom_fail(char *err, size_t errlen, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, errlen, fmt, ap);
    va_end(ap);
    return TG_ERR_ARG;
}

int tg::build_geom(const tg_config &c, Geom &g, char *err, size_t errlen) {
    memset(&g, 0, sizeof g);
    if (c.dims != 2 && c.dims != 3) return geom_fail(err, errlen, "dims must be 2 or 3 (got %d)", c.dims);
    if (c.order < 1 || c.order > 3) return geom_fail(err, errlen, "order must be 1, 2 or 3 (got %d)", c.order);
    const int ng_expect = c.order == 1 ? 5 : 7;
    if (c.nghost != ng_expect)
        return geom_fail(err, errlen, "nghost must be %d for order %d (got %d)", ng_expect, c.order, c.nghost);
    if (c.dims == 2 && (c.mz != 1 || c.nghostz != 5))
        return geom_fail(err, errlen, "2D needs mz = 1 and nghostz = 5");
    if (c.dims == 3 && c.nghostz != c.nghost) return geom_fail(err, errlen, "3D needs nghostz = nghost");
    g.dims = c.dims;
    g.order = c.order;
    g.mx = c.mx;
    g.my = c.my;
    g.mz = c.mz;
    g.ng = c.nghost;
    g.ngz = c.nghostz;
    const int nx = c.mx - g.ng, ny = c.my - g.ng, nz = c.dims == 3 ? c.mz - g.ngz : 1;
    // more interior cells per axis than half the ghost band (nghost/2 + 1:
    // 3 at order 1, 4 at orders 2 and 3): below that the periodic images of
    // the ghost layers are themselves ghost layers, and the current fold's
    // first slab would read cells it writes
    const int nmin = g.ng / 2 + 1, nzmin = c.dims == 3 ? g.ngz / 2 + 1 : 1;
    if (nx < nmin || ny < nmin || nz < nzmin)
        return geom_fail(err, errlen, "grid too small (%d x %d x %d interior cells; at least %d per axis)", nx, ny,
                         nz, nmin);
    g.lot = (long long)c.mx * c.my * c.mz;
    if (g.lot >= (1LL << 31)) return geom_fail(err, errlen, "grid of %lld cells exceeds int32 cell indices", g.lot);
    g.sy = c.mx;
    g.sz = (long long)c.mx * c.my;
    for (int a = 0; a < 3; a++) g.per[a] = c.periodic[a] ? 1 : 0;
    if (c.dims == 2) g.per[2] = 0;
    g.minx = (float)(g.ng / 2 + 1);
    g.maxx = (float)c.mx - 1.0f * (float)(g.ng / 2);
    g.miny = (float)(g.ng / 2 + 1);
    g.maxy = (float)c.my - 1.0f * (float)(g.ng / 2);
    if (c.dims == 3) {
        g.minz = 1.0f * (float)(g.ngz / 2 + 1);
        g.maxz = (float)c.mz - 1.0f * (float)(g.ngz / 2);
    } else {
        g.minz = 1.0f * (float)(g.ngz / 2 + 1);
        g.maxz = 1.0f * (float)(g.ngz / 2 + 1) + 1.0f;
    }
    // tiles
    int tx = c.tile[0], ty = c.tile[1], tz = c.tile[2];
    if (tx <= 0) tx = c.dims == 3 ? 8 : 16;
    if (ty <= 0) ty = c.dims == 3 ? 8 : 16;
    if (tz <= 0) tz = c.dims == 3 ? 8 : 1;
    if (c.dims == 2) tz = 1;
    g.tx = tx;
    g.ty = ty;
    g.tz = tz;
    g.ox = g.ng / 2 + 1;
    g.oy = g.ng / 2 + 1;
    g.oz = c.dims == 3 ? g.ngz / 2 + 1 : 1;
    g.ntx = (nx + tx - 1) / tx;
    g.nty = (ny + ty - 1) / ty;
    g.ntz = c.dims == 3 ? (nz + tz - 1) / tz : 1;
    g.ntiles = g.ntx * g.nty * g.ntz;
    // The deposit stencil of a particle whose lap starts in cell i spans
    // cells [i - 2, i + 3] (shape orders 2 and 3; [i - 1, i + 2] for order
    // 1). A sort leaves every particle in its tile, and between sorts a
    // particle moves less than c cells per lap, so the window covers the
    // tile, the stencil and the drift of the laps since the last sort.
    const int se = c.sort_every < 1 ? 1 : c.sort_every;
#ifndef TG_HALO_EXTRA
#define TG_HALO_EXTRA 0
#endif
    const int drift = TG_HALO_EXTRA + (int)ceilf((float)(se - 1) * c.c);
    g.wlo = (c.order == 1 ? 1 : 2) + drift;
    g.whi = (c.order == 1 ? 2 : 3) + drift;
    g.wx = tx + g.wlo + g.whi;
    g.wy = ty + g.wlo + g.whi;
    g.wz = c.dims == 3 ? tz + g.wlo + g.whi : 1;
    g.wcells = g.wx * g.wy * g.wz;
    // 3D field copy over the gather's reach (nodes [i - 1, i + 2] of a
    // particle starting in cell i, widened by the drift), kept only while two
    // CTAs per SM fit beside the deposit window
    g.fw_lo = g.fwx = g.fwy = g.fwz = g.fwcells = 0;
    if (c.dims == 3) {
        const int drift_cells = g.wlo - (c.order == 1 ? 1 : 2);
        g.fw_lo = drift_cells + 1;
        g.fwx = tx + 2 * drift_cells + 3;
        g.fwy = ty + 2 * drift_cells + 3;
        g.fwz = tz + 2 * drift_cells + 3;
        g.fwcells = g.fwx * g.fwy * g.fwz;
        if (tile_smem_bytes(3, g.wcells, g.fwcells) > 112 * 1024) g.fw_lo = g.fwx = g.fwy = g.fwz = g.fwcells = 0;
    }
    const size_t smem = tile_smem_bytes(c.dims, g.wcells, g.fwcells);  // window and field copy
    if (smem > 227 * 1024)
        return geom_fail(err, errlen, "tile shared memory (deposit window and field copy) of %zu bytes exceeds 227 KB; use smaller tiles", smem);
    return TG_OK;
}

void tg::build_params(const tg_config &c, Params &P) {
    memset(&P, 0, sizeof P);
    P.c = c.c;
    P.corr = c.corr;
    P.qm[0] = c.qmi;
    P.qm[1] = c.qme;
    P.qs[0] = c.qi;
    P.qs[1] = c.qe;
    P.external_fields = c.external_fields;
    for (int a = 0; a < 6; a++) P.ext[a] = c.ext[a];
    P.x1in = c.x1in; P.x2in = c.x2in; P.y1in = c.y1in; P.y2in = c.y2in; P.z1in = c.z1in; P.z2in = c.z2in;
    P.mxcum = c.mxcum; P.mycum = c.mycum; P.mzcum = c.mzcum;
    P.fixed = c.deposit_mode == TG_DEPOSIT_FIXED;
    P.fx_scale = ldexpf(1.0f, c.fx_shift);
    P.fx_inv = ldexp(1.0, -c.fx_shift);
    P.quirks = c.quirks;
}

static int setup_geom(tg_ctx *ctx) { return build_geom(ctx->cfg, ctx->g, ctx->err, sizeof ctx->err); }

static void setup_params(tg_ctx *ctx) { build_params(ctx->cfg, ctx->P); }

static int alloc_species(tg_ctx *ctx, Species &s, size_t n) {
    int r;
    if ((r = dalloc(ctx, &s.cell, n))) return r;
    if ((r = dalloc(ctx, &s.ox, n))) return r;
    if ((r = dalloc(ctx, &s.oy, n))) return r;
    if ((r = dalloc(ctx, &s.oz, n))) return r;
    if ((r = dalloc(ctx, &s.u, n))) return r;
    if ((r = dalloc(ctx, &s.v, n))) return r;
    if ((r = dalloc(ctx, &s.w, n))) return r;
    if ((r = dalloc(ctx, &s.ch, n))) return r;
    if ((r = dalloc(ctx, &s.ind, n))) return r;
    if ((r = dalloc(ctx, &s.proc, n))) return r;
    if ((r = dalloc(ctx, &s.splitlev, n))) return r;
    return TG_OK;
}

extern "C" int tg_init(const tg_config *cfg, tg_ctx **out) {
    if (!cfg || !out) return fail(nullptr, TG_ERR_ARG, "tg_init: null argument");
    *out = nullptr;
    tg_ctx *ctx = new (std::nothrow) tg_ctx();
    if (!ctx) return fail(nullptr, TG_ERR_ARG, "tg_init: out of host memory");
    ctx->cfg = *cfg;
    int r = setup_geom(ctx);
    if (r) {
        fail(nullptr, r, "%s", ctx->err);
        delete ctx;
        return r;
    }
    setup_params(ctx);
    if (cfg->maxhlf <= 0 || cfg->maxhlf >= (1LL << 31)) {
        delete ctx;
        return fail(nullptr, TG_ERR_ARG, "maxhlf must be in [1, 2^31)");
    }
    ctx->device = cfg->device;
    cudaError_t e = cudaSetDevice(cfg->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        fail(nullptr, TG_ERR_CUDA, "tg_init: CUDA device %d unavailable: %s", cfg->device, cudaGetErrorString(e));
        delete ctx;
        return TG_ERR_CUDA;
    }
    const Geom &g = ctx->g;
    const size_t lot = (size_t)g.lot;
    r = TG_OK;
    for (int a = 0; a < 9 && !r; a++) r = dalloc(ctx, &ctx->f[a], lot);
    for (int a = 0; a < 3 && !r; a++) r = dalloc(ctx, &ctx->ftmp[a], lot);
    if (g.dims == 3)
        r = dalloc(ctx, &ctx->prim, 2 * lot);
    if (ctx->P.fixed)
        for (int a = 0; a < 3 && !r; a++) r = dalloc(ctx, &ctx->fix[a], lot);
    for (int p = 0; p < 2 && !r; p++)
        for (int s = 0; s < 2 && !r; s++) r = alloc_species(ctx, ctx->sp[p][s], (size_t)cfg->maxhlf);
    if (!r) r = dalloc(ctx, &ctx->d_cnt, 4);
    for (int s = 0; s < 2 && !r; s++) {
        r = dalloc(ctx, &ctx->tstart[s], (size_t)g.ntiles + 1);
        if (!r) r = dalloc(ctx, &ctx->hist[s], (size_t)g.ntiles);
        if (!r) r = dalloc(ctx, &ctx->cursor[s], (size_t)g.ntiles);
    }
    if (!r) r = dalloc(ctx, &ctx->d_status, 1);
    if (!r) r = dalloc(ctx, &ctx->d_dead, 1);
    {
        const size_t nint = (size_t)(g.mx - g.ng) * (g.my - g.ng) * (g.dims == 3 ? g.mz - g.ngz : 1);
        if (!r) r = dalloc(ctx, &ctx->rhofx, nint);
        if (!r) r = dalloc(ctx, &ctx->rho[0], nint);
        if (!r) r = dalloc(ctx, &ctx->rho[1], nint);
        if (!r) r = dalloc(ctx, &ctx->dacc, 16);
        if (!r) r = dalloc(ctx, &ctx->dhist, (size_t)ctx->hist_cap * 16);
        if (!r) r = dalloc(ctx, &ctx->dcounter, 1);
        if (!r) {
            e = cudaMemsetAsync(ctx->rhofx, 0, nint * 8, ctx->st);
            if (e == cudaSuccess) e = cudaMemsetAsync(ctx->dacc, 0, 16 * 8, ctx->st);
            if (e == cudaSuccess) e = cudaMemsetAsync(ctx->dhist, 0, (size_t)ctx->hist_cap * 16 * 8, ctx->st);
            if (e == cudaSuccess) e = cudaMemsetAsync(ctx->dcounter, 0, 8, ctx->st);
        }
    }
    if (r) {
        snprintf(g_init_error, sizeof g_init_error, "%s", ctx->err);
        tg_finalize(ctx);
        return r;
    }
    cudaStream_t st = ctx->st;
    for (int a = 0; a < 9; a++) e = e != cudaSuccess ? e : cudaMemsetAsync(ctx->f[a], 0, lot * 4, st);
    for (int a = 0; a < 3; a++) e = e != cudaSuccess ? e : cudaMemsetAsync(ctx->ftmp[a], 0, lot * 4, st);
    if (ctx->P.fixed)
        for (int a = 0; a < 3; a++) e = e != cudaSuccess ? e : cudaMemsetAsync(ctx->fix[a], 0, lot * 8, st);
    for (int s = 0; s < 2; s++) {
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->tstart[s], 0, ((size_t)g.ntiles + 1) * 4, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->hist[s], 0, (size_t)g.ntiles * 4, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->cursor[s], 0, (size_t)g.ntiles * 4, st);
    }
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_cnt, 0, 4 * sizeof(long long), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_status, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_dead, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        fail(nullptr, TG_ERR_CUDA, "tg_init: %s", cudaGetErrorString(e));
        tg_finalize(ctx);
        return TG_ERR_CUDA;
    }
    *out = ctx;
    return TG_OK;
}

extern "C" void tg_finalize(tg_ctx *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->st) cudaStreamSynchronize(ctx->st);
    for (int p = 0; p < 2; p++)
        if (ctx->cycle[p]) cudaGraphExecDestroy(ctx->cycle[p]);
    for (auto &e : ctx->ev) cudaEventDestroy(e);
    for (void *q : ctx->allocs) cudaFree(q);
    if (ctx->stage) cudaFree(ctx->stage);
    if (ctx->stage2) cudaFree(ctx->stage2);
    for (int a = 0; a < 4; a++)
        if (ctx->rk[a]) cudaFree(ctx->rk[a]);
    if (ctx->cub_tmp) cudaFree(ctx->cub_tmp);
    for (auto &e : ctx->ev_link)
        if (e) cudaEventDestroy(e);
    for (void *h : ctx->pinned) cudaHostUnregister(h);
    if (ctx->st_up) cudaStreamDestroy(ctx->st_up);
    if (ctx->st_down) cudaStreamDestroy(ctx->st_down);
    if (ctx->st) cudaStreamDestroy(ctx->st);
    delete ctx;
}

extern "C" const char *tg_last_error(tg_ctx *ctx) { return ctx ? ctx->err : g_init_error; }

// error text for entry points that have no context (tg_last_error(NULL))
void tg::tg_set_global_error(const char *msg) { snprintf(g_init_error, sizeof g_init_error, "%s", msg); }

extern "C" int tg_synchronize(tg_ctx *ctx) {
    if (!ctx) return TG_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->st));
    return check_status(ctx);
}

extern "C" void *tg_stream(tg_ctx *ctx) { return ctx ? (void *)ctx->st : nullptr; }

extern "C" int tg_device_fields(tg_ctx *ctx, float **ptrs9) {
    if (!ctx || !ptrs9) return TG_ERR_ARG;
    for (int a = 0; a < 9; a++) ptrs9[a] = ctx->f[a];
    return TG_OK;
}

extern "C" int32_t tg_kernels_per_step(tg_ctx *ctx) { return ctx ? ctx->kernels_per_step : 0; }

// ---------------------------------------------------------------------------
// tile sort: count (unless the tile kernel already did), scan, scatter,
// flip parity
// ---------------------------------------------------------------------------
// grid-size hint for kernels that read the particle count on the device:
// the host's count, or the capacity when device-side injection may have
// grown it since
static long long count_hint(const tg_ctx *ctx, int s) {
    return ctx->shock_on ? (long long)ctx->cfg.maxhlf : ctx->hcount[s];
}

static int sort_species(tg_ctx *ctx, int s, bool counted) {
    const int p = ctx->par;
    long long *cnt_cur = ctx->d_cnt + 2 * p + s, *cnt_next = ctx->d_cnt + 2 * (1 - p) + s;
    if (!counted) CK(launch_tile_count(ctx->g, ctx->sp[p][s], cnt_cur, count_hint(ctx, s), ctx->hist[s], ctx->st));
    CK(launch_scan(ctx->hist[s], ctx->tstart[s], ctx->cursor[s], ctx->g.ntiles, cnt_next, ctx->st));
    CK(launch_scatter(ctx->g, ctx->sp[p][s], ctx->sp[1 - p][s], cnt_cur, count_hint(ctx, s), ctx->tstart[s],
                      ctx->cursor[s], ctx->st));
    return TG_OK;
}

static int sort_all(tg_ctx *ctx, bool counted) {
    int r;
    if ((r = sort_species(ctx, 0, counted))) return r;
    if ((r = sort_species(ctx, 1, counted))) return r;
    CK(cudaMemsetAsync(ctx->d_dead, 0, sizeof(int), ctx->st));
    ctx->fault_seen = false;
    ctx->par ^= 1;
    ctx->dirty = false;
    ctx->may_have_dead = false;
    return TG_OK;
}

static int ensure_sorted(tg_ctx *ctx) {
    if (!ctx->dirty) return TG_OK;
    return sort_all(ctx, false);
}

// The overlapped host-driven lap (tg_step_host): the records of each species
// travel by DMA (copy engines, no SMs) between the page-locked host array and
// a device staging copy of it, in parts of consecutive records; each part is
// converted and tile-sorted on its own as soon as its records are in, pushed
// by its own tile launch, converted back and sent home while later parts are
// still arriving and the field phases run. Part h of species s holds records
// [off[s][h], off[s][h+1]) in the host array, the staging copy and both
// particle parities.
struct HostPipe {
    char *host;             // the bound host records
    char *stage;            // device staging copy, same layout
    cudaStream_t down;      // device -> host copies
    int parts;
    long long off[2][TG_HOST_PARTS_MAX + 1];
    cudaEvent_t uploaded[2][TG_HOST_PARTS_MAX], pushed[2][TG_HOST_PARTS_MAX];
    int *ts[2][TG_HOST_PARTS_MAX];  // tile starts per part (written by the part's scan)
};

// the records [o, ...) of a species as a species of their own
static Species species_at(const Species &s, long long o) {
    Species v = s;
    v.cell += o;
    v.ox += o;
    v.oy += o;
    v.oz += o;
    v.u += o;
    v.v += o;
    v.w += o;
    v.ch += o;
    v.ind += o;
    v.proc += o;
    v.splitlev += o;
    return v;
}

static TileArgs tile_args(tg_ctx *ctx, bool count_tiles) {
    TileArgs a;
    memset(&a, 0, sizeof a);
    a.g = ctx->g;
    a.P = ctx->P;
    a.f.ex = ctx->f[0]; a.f.ey = ctx->f[1]; a.f.ez = ctx->f[2];
    a.f.bx = ctx->f[3]; a.f.by = ctx->f[4]; a.f.bz = ctx->f[5];
    a.f.prim = ctx->prim;
    for (int s = 0; s < 2; s++) {
        a.sp[s] = ctx->sp[ctx->par][s];
        a.tstart[s] = ctx->tstart[s];
        a.newcount[s] = count_tiles ? ctx->hist[s] : nullptr;
    }
    for (int cc = 0; cc < 3; cc++) {
        a.cur[cc] = ctx->f[6 + cc];
        a.fix[cc] = ctx->fix[cc];
    }
    a.status = ctx->d_status;
    a.dead = ctx->d_dead;
    if (ctx->shock_on) {
        a.shock = ctx->d_shock;
        a.wall = ctx->K.wall;
        a.gammawall = ctx->K.gammawall;
        a.betawall = ctx->K.betawall;
    }
    return a;
}

// ---------------------------------------------------------------------------
// bindings and host transfers
// ---------------------------------------------------------------------------
extern "C" int tg_bind_fields(tg_ctx *ctx, float *ex, float *ey, float *ez, float *bx, float *by, float *bz,
                              float *curx, float *cury, float *curz) {
    if (!ctx) return TG_ERR_ARG;
    float *h[9] = {ex, ey, ez, bx, by, bz, curx, cury, curz};
    for (int a = 0; a < 9; a++) ctx->hf[a] = h[a];
    return TG_OK;
}

extern "C" int tg_bind_particles(tg_ctx *ctx, void *p, int32_t *ions, int32_t *lecs) {
    if (!ctx || !p || !ions || !lecs) return fail(ctx, TG_ERR_ARG, "tg_bind_particles: null argument");
    ctx->hp = p;
    ctx->hions = ions;
    ctx->hlecs = lecs;
    return TG_OK;
}

static const size_t AOS = 40;

// A device-usable view of a page-locked (registered or pinned) host array:
// its device pointer, so the conversion kernels read and write the records
// in place at the link's bandwidth; NULL for pageable memory (staged copies
// are used then: a kernel walking pageable memory through the host page
// tables is far slower than a staged copy).
static void *host_view(tg_ctx *ctx, void *h) {
    (void)ctx;
    if ((uintptr_t)h & 7) return nullptr;  // the conversion kernels move 8-byte words
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, h) == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer)
        return at.devicePointer;
    (void)cudaGetLastError();
    return nullptr;
}

extern "C" int tg_sync_from_host(tg_ctx *ctx, unsigned mask) {
    TG_RANGE("tg_sync_from_host");
    if (!ctx) return TG_ERR_ARG;
    const size_t lot = (size_t)ctx->g.lot;
    const int groups[3][4] = {{0, 1, 2, (int)TG_SYNC_E}, {3, 4, 5, (int)TG_SYNC_B}, {6, 7, 8, (int)TG_SYNC_CUR}};
    for (int gi = 0; gi < 3; gi++) {
        if (!(mask & (unsigned)groups[gi][3])) continue;
        for (int a = 0; a < 3; a++) {
            float *h = ctx->hf[groups[gi][a]];
            if (!h) return fail(ctx, TG_ERR_STATE, "tg_sync_from_host: field array %d not bound", groups[gi][a]);
            CK(cudaMemcpyAsync(ctx->f[groups[gi][a]], h, lot * 4, cudaMemcpyHostToDevice, ctx->st));
        }
    }
    if (mask & TG_SYNC_PARTICLES) {
        if (!ctx->hp) return fail(ctx, TG_ERR_STATE, "tg_sync_from_host: particles not bound");
        const long long n[2] = {*ctx->hions, *ctx->hlecs};
        for (int s = 0; s < 2; s++)
            if (n[s] < 0 || n[s] > ctx->cfg.maxhlf)
                return fail(ctx, TG_ERR_OVERFLOW, "species %d count %lld outside [0, maxhlf=%lld]", s, n[s],
                            (long long)ctx->cfg.maxhlf);
        const char *hbase = (const char *)host_view(ctx, ctx->hp);
        if (!hbase && !ctx->stage) CK(cudaMalloc(&ctx->stage, (size_t)ctx->cfg.maxhlf * AOS + 256));
        for (int s = 0; s < 2; s++) {
            const size_t off = s == 0 ? 0 : (size_t)ctx->cfg.maxhlf * AOS;
            if (hbase) {
                // the conversion kernel reads the host records directly
                CK(launch_aos_to_soa(ctx->g, hbase + off, ctx->sp[ctx->par][s], n[s], ctx->d_status, ctx->st));
            } else {
                const char *src = (const char *)ctx->hp + off;
                CK(cudaMemcpyAsync(ctx->stage, src, (size_t)n[s] * AOS, cudaMemcpyHostToDevice, ctx->st));
                CK(launch_aos_to_soa(ctx->g, ctx->stage, ctx->sp[ctx->par][s], n[s], ctx->d_status, ctx->st));
            }
            CK(cudaMemcpyAsync(ctx->d_cnt + 2 * ctx->par + s, &n[s], sizeof(long long), cudaMemcpyHostToDevice,
                               ctx->st));
            ctx->hcount[s] = n[s];
        }
        CK(cudaStreamSynchronize(ctx->st));  // n[] lives on this stack frame
        ctx->dirty = true;
        ctx->may_have_dead = true;  // records outside the grid were dropped
    }
    return TG_OK;
}

// current counts of the buffer in use (drops discarded particles first; the
// order of a buffer without discarded entries is left as it is)
static int exact_counts(tg_ctx *ctx, long long n[2]) {
    if (ctx->may_have_dead) {
        // dropped entries exist only after a deliberate drop or a reported
        // fault; otherwise the buffer is already compact
        int flags[2] = {1, 1};
        CK(cudaMemcpyAsync(&flags[0], ctx->d_dead, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaMemcpyAsync(&flags[1], ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        if (flags[0] != 0 || flags[1] != 0 || ctx->fault_seen) {
            int r = sort_all(ctx, false);
            if (r) return r;
        } else {
            ctx->may_have_dead = false;
        }
    }
    CK(cudaMemcpyAsync(n, ctx->d_cnt + 2 * ctx->par, 2 * sizeof(long long), cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->hcount[0] = n[0];
    ctx->hcount[1] = n[1];
    return TG_OK;
}

extern "C" int tg_get_counts(tg_ctx *ctx, int64_t *ions, int64_t *lecs) {
    if (!ctx) return TG_ERR_ARG;
    long long n[2];
    int r = exact_counts(ctx, n);
    if (r) return r;
    if (ions) *ions = n[0];
    if (lecs) *lecs = n[1];
    return check_status(ctx);
}

extern "C" int tg_sync_to_host(tg_ctx *ctx, unsigned mask) {
    TG_RANGE("tg_sync_to_host");
    if (!ctx) return TG_ERR_ARG;
    const size_t lot = (size_t)ctx->g.lot;
    const int groups[3][4] = {{0, 1, 2, (int)TG_SYNC_E}, {3, 4, 5, (int)TG_SYNC_B}, {6, 7, 8, (int)TG_SYNC_CUR}};
    for (int gi = 0; gi < 3; gi++) {
        if (!(mask & (unsigned)groups[gi][3])) continue;
        for (int a = 0; a < 3; a++) {
            float *h = ctx->hf[groups[gi][a]];
            if (!h) return fail(ctx, TG_ERR_STATE, "tg_sync_to_host: field array %d not bound", groups[gi][a]);
            CK(cudaMemcpyAsync(h, ctx->f[groups[gi][a]], lot * 4, cudaMemcpyDeviceToHost, ctx->st));
        }
    }
    if (mask & TG_SYNC_PARTICLES) {
        if (!ctx->hp) return fail(ctx, TG_ERR_STATE, "tg_sync_to_host: particles not bound");
        long long n[2];
        int r = exact_counts(ctx, n);
        if (r) return r;
        char *hbase = (char *)host_view(ctx, ctx->hp);
        if (!hbase && !ctx->stage) CK(cudaMalloc(&ctx->stage, (size_t)ctx->cfg.maxhlf * AOS + 256));
        for (int s = 0; s < 2; s++) {
            const size_t off = s == 0 ? 0 : (size_t)ctx->cfg.maxhlf * AOS;
            if (hbase) {
                // the conversion kernel writes the host records directly
                CK(launch_soa_to_aos(ctx->g, ctx->sp[ctx->par][s], hbase + off, n[s], ctx->st));
            } else {
                char *dst = (char *)ctx->hp + off;
                CK(launch_soa_to_aos(ctx->g, ctx->sp[ctx->par][s], ctx->stage, n[s], ctx->st));
                CK(cudaMemcpyAsync(dst, ctx->stage, (size_t)n[s] * AOS, cudaMemcpyDeviceToHost, ctx->st));
                CK(cudaStreamSynchronize(ctx->st));
            }
        }
        *ctx->hions = (int32_t)n[0];
        *ctx->hlecs = (int32_t)n[1];
    }
    CK(cudaStreamSynchronize(ctx->st));
    return check_status(ctx);
}

// ---------------------------------------------------------------------------
// per-subroutine entry points
// ---------------------------------------------------------------------------
extern "C" int tg_bc_b1(tg_ctx *ctx) {
    TG_RANGE("bc_b1");
    if (!ctx) return TG_ERR_ARG;
    CK(launch_ghost(ctx->g, ctx->f[3], ctx->f[4], ctx->f[5], GHOST_BC, ctx->st));
    return TG_OK;
}

extern "C" int tg_bc_e1(tg_ctx *ctx) {
    TG_RANGE("bc_e1");
    if (!ctx) return TG_ERR_ARG;
    CK(launch_ghost(ctx->g, ctx->f[0], ctx->f[1], ctx->f[2], GHOST_BC, ctx->st));
    return TG_OK;
}

extern "C" int tg_advance_b_half(tg_ctx *ctx) {
    TG_RANGE("advance_Bhalfstep");
    if (!ctx) return TG_ERR_ARG;
    CK(launch_advance_b(ctx->g, ctx->P, ctx->f, ctx->st));
    return TG_OK;
}

extern "C" int tg_advance_e(tg_ctx *ctx) {
    TG_RANGE("advance_Efield");
    if (!ctx) return TG_ERR_ARG;
    CK(launch_advance_e(ctx->g, ctx->P, ctx->f, ctx->st));
    return TG_OK;
}

extern "C" int tg_move(tg_ctx *ctx) {
    TG_RANGE("move_particles");
    if (!ctx) return TG_ERR_ARG;
    FieldPtrs fp;
    fp.ex = ctx->f[0]; fp.ey = ctx->f[1]; fp.ez = ctx->f[2];
    fp.bx = ctx->f[3]; fp.by = ctx->f[4]; fp.bz = ctx->f[5];
    fp.prim = ctx->prim;
    if (ctx->g.dims == 3) CK(launch_primal(ctx->g, ctx->f, ctx->prim, ctx->st));
    for (int s = 0; s < 2; s++)
        CK(launch_push_flat(ctx->g, ctx->P, fp, ctx->sp[ctx->par][s], ctx->d_cnt + 2 * ctx->par + s,
                            count_hint(ctx, s), ctx->P.qm[s], ctx->d_status, ctx->st));
    ctx->dirty = true;
    ctx->may_have_dead = true;
    return TG_OK;
}

extern "C" int tg_reset_currents(tg_ctx *ctx) {
    TG_RANGE("reset_currents");
    if (!ctx) return TG_ERR_ARG;
    const size_t lot = (size_t)ctx->g.lot;
    for (int a = 6; a < 9; a++) CK(cudaMemsetAsync(ctx->f[a], 0, lot * 4, ctx->st));
    return TG_OK;
}

extern "C" int tg_deposit(tg_ctx *ctx) {
    TG_RANGE("deposit_particles");
    if (!ctx) return TG_ERR_ARG;
    int r = ensure_sorted(ctx);
    if (r) return r;
    TileArgs a = tile_args(ctx, false);
    CK(launch_tiles(a, ctx->P.fixed != 0, false, true, ctx->st));
    if (ctx->P.fixed) {
        // cur = the fixed-point sum since reset_currents (which it follows)
        float *cur3[3] = {ctx->f[6], ctx->f[7], ctx->f[8]};
        CK(launch_fixed_to_float(ctx->g, ctx->P, ctx->fix, cur3, ctx->st));
    }
    ctx->dirty = true;  // wrapped particles left their tiles
    ctx->may_have_dead = true;
    return TG_OK;
}

extern "C" int tg_fold_currents(tg_ctx *ctx) {
    TG_RANGE("exchange_current");
    if (!ctx) return TG_ERR_ARG;
    CK(launch_fold(ctx->g, ctx->P, ctx->f + 6, ctx->st));
    return TG_OK;
}

static int filter_passes(tg_ctx *ctx) {
    float *a[3] = {ctx->f[6], ctx->f[7], ctx->f[8]};
    float *b[3] = {ctx->ftmp[0], ctx->ftmp[1], ctx->ftmp[2]};
    for (int n = 0; n < ctx->cfg.ntimes; n++) {
        if (n % 2 == 0) CK(launch_filter_pass(ctx->g, a, b, ctx->st));
        else CK(launch_filter_pass(ctx->g, b, a, ctx->st));
    }
    if (ctx->cfg.ntimes % 2 == 1)
        for (int cc = 0; cc < 3; cc++)
            CK(cudaMemcpyAsync(a[cc], b[cc], (size_t)ctx->g.lot * 4, cudaMemcpyDeviceToDevice, ctx->st));
    return TG_OK;
}

extern "C" int tg_filter(tg_ctx *ctx) {
    TG_RANGE("apply_filter1_opt");
    if (!ctx) return TG_ERR_ARG;
    return filter_passes(ctx);
}

extern "C" int tg_add_current(tg_ctx *ctx) {
    TG_RANGE("add_current");
    if (!ctx) return TG_ERR_ARG;
    CK(launch_add_current(ctx->g, ctx->f, ctx->st));
    return TG_OK;
}

extern "C" int tg_reorder(tg_ctx *ctx, int32_t lap, int32_t force) {
    TG_RANGE("reorder_particles");
    if (!ctx) return TG_ERR_ARG;
    if (!force) {
        // code/particles.F90:398-400
        if (lap == ctx->lapreorder + 1) return TG_OK;
        if (lap % 10 != 0) return TG_OK;
    }
    long long n[2];
    int r = exact_counts(ctx, n);
    if (r) return r;
    const size_t cap = (size_t)ctx->cfg.maxhlf;
    for (int a = 0; a < 4; a++)
        if (!ctx->rk[a]) CK(cudaMalloc(&ctx->rk[a], cap * 4 + 256));
    const long long maxkey = (long long)ctx->g.lot + ctx->g.sy + ctx->g.sz + ctx->g.mx + 1;
    int end_bit = 1;
    while ((1LL << end_bit) <= maxkey) end_bit++;
    if (!ctx->cub_tmp) {
        CK(cub::DeviceRadixSort::SortPairs(nullptr, ctx->cub_bytes, ctx->rk[0], ctx->rk[1], ctx->rk[2], ctx->rk[3],
                                           (int)cap, 0, end_bit, ctx->st));
        CK(cudaMalloc(&ctx->cub_tmp, ctx->cub_bytes + 256));
    }
    const int p = ctx->par;
    for (int s = 0; s < 2; s++) {
        CK(launch_reorder_keys(ctx->g, ctx->sp[p][s], n[s], ctx->rk[0], ctx->rk[2], ctx->st));
        size_t bytes = ctx->cub_bytes;
        // stable LSD radix sort by the reference's cell key (library sort,
        // off the per-lap path)
        CK(cub::DeviceRadixSort::SortPairs(ctx->cub_tmp, bytes, ctx->rk[0], ctx->rk[1], ctx->rk[2], ctx->rk[3],
                                           (int)n[s], 0, end_bit, ctx->st));
        CK(launch_gather(ctx->sp[p][s], ctx->sp[1 - p][s], ctx->rk[3], n[s], ctx->st));
        CK(cudaMemcpyAsync(ctx->d_cnt + 2 * (1 - p) + s, ctx->d_cnt + 2 * p + s, sizeof(long long),
                           cudaMemcpyDeviceToDevice, ctx->st));
    }
    ctx->par ^= 1;
    ctx->dirty = true;  // grouped by cell, not by tile
    ctx->lapreorder = lap;
    return TG_OK;
}

// ---------------------------------------------------------------------------
// FP64 diagnostics
// ---------------------------------------------------------------------------
// pipe: the particles are grouped by tile part by part (a host-driven lap)
// the diagnostics' launch descriptor over the particle buffers in use
static DiagLaunch diag_launch(tg_ctx *ctx) {
    DiagLaunch d;
    memset(&d, 0, sizeof d);
    d.g = ctx->g;
    d.P = ctx->P;
    for (int s = 0; s < 2; s++) {
        d.sp[s] = ctx->sp[ctx->par][s];
        d.tstart[s] = ctx->tstart[s];
        d.mass[s] = fabsf(ctx->P.qs[s] / ctx->P.qm[s]);
    }
    for (int a = 0; a < 6; a++) d.f[a] = ctx->f[a];
    d.rhofx = ctx->rhofx;
    d.rho[0] = ctx->rho[0];
    d.rho[1] = ctx->rho[1];
    d.acc = ctx->dacc;
    d.hist = ctx->dhist;
    d.hist_cap = ctx->hist_cap;
    d.counter = ctx->dcounter;
    d.ntimes = ctx->cfg.ntimes;
    d.status = ctx->d_status;
    return d;
}

// the lap's diagnostics; particles = false when the particle pass already
// ran (part by part inside a host-driven lap)
static int run_diag(tg_ctx *ctx, bool particles) {
    DiagLaunch d = diag_launch(ctx);
    d.particles = particles;
    CK(launch_diag(d, ctx->st));
    return TG_OK;
}

void tg::record_to_diag(const double *h, tg_diag *out) {
    memset(out, 0, sizeof *out);
    out->gauss_abs = sqrt(h[0]);
    out->rho_norm = sqrt(h[1]);
    out->gauss_residual = h[1] > 0.0 ? sqrt(h[0] / h[1]) : sqrt(h[0]);
    out->charge_total = h[2];
    out->e_field = h[3];
    out->e_mag = h[4];
    out->e_kin_ions = h[5];
    out->e_kin_lecs = h[6];
    for (int a = 0; a < 3; a++) {
        out->p_part[a] = h[7 + a];
        out->p_field[a] = h[10 + a];
    }
}

extern "C" int tg_diag_history(tg_ctx *ctx, double *out, int32_t n) {
    if (!ctx || !out || n < 0) return TG_ERR_ARG;
    unsigned long long cnt = 0;
    CK(cudaMemcpyAsync(&cnt, ctx->dcounter, 8, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    long long have = (long long)cnt < ctx->hist_cap ? (long long)cnt : ctx->hist_cap;
    if (n > have) n = (int32_t)have;
    for (int32_t r = 0; r < n; r++) {
        const unsigned long long idx = (cnt - (unsigned long long)n + (unsigned long long)r) % (unsigned long long)ctx->hist_cap;
        CK(cudaMemcpyAsync(out + (size_t)r * 16, ctx->dhist + idx * 16, 16 * 8, cudaMemcpyDeviceToHost, ctx->st));
    }
    CK(cudaStreamSynchronize(ctx->st));
    return n;
}

// ---------------------------------------------------------------------------
// collisionless-shock hooks
// ---------------------------------------------------------------------------
static const int INJECT_GRID = 152 * 4;

// init_maxw_table (code/particles.F90:2126-2163) on the host, as the
// reference evaluates it (single precision, sequential sums, normalised by
// the element pdf_sz read before the assignment)
static void maxw_table(float delgam, int dims, float pcosthmult, float *gt, float *pt) {
    const float maxg = delgam * 20.0f + 1.0f;
    std::vector<float> func(TG_PDF_SZ);
    for (int i = 1; i <= TG_PDF_SZ; i++) gt[i - 1] = (maxg - 1.0f) / (float)(TG_PDF_SZ - 1) * (float)(i - 1);
    for (int i = 0; i < TG_PDF_SZ; i++) {
        const float g = gt[i];
        if (dims == 3 || pcosthmult == 1.0f) func[i] = (g + 1.0f) * sqrtf(g * (g + 2.0f)) * expf(-g / delgam);
        else func[i] = (g + 1.0f) * expf(-g / delgam);
    }
    pt[0] = 0.0f;
    float sum = 0.0f;
    for (int i = 1; i <= TG_PDF_SZ; i++) {
        sum = sum + func[i - 1];
        pt[i] = sum;
    }
    const float norm = pt[TG_PDF_SZ - 1];
    for (int i = 0; i <= TG_PDF_SZ; i++) pt[i] = pt[i] / norm;
}

static long long host_powmod31(long long a, long long e) {
    unsigned long long r = 1, b = (unsigned long long)a;
    while (e > 0) {
        if (e & 1) r = (r * b) % 2147483647ULL;
        b = (b * b) % 2147483647ULL;
        e >>= 1;
    }
    return (long long)r;
}

extern "C" int tg_shock_init(tg_ctx *ctx, const tg_shock *k) {
    if (!ctx || !k) return TG_ERR_ARG;
    if (ctx->g.dims != 2) return fail(ctx, TG_ERR_ARG, "tg_shock_init: the shock hooks are 2D");
    // between sorts the injected particles sit past the tile ranges: the tail
    // kernel moves them, but the tile-wise diagnostics pass would miss them
    if (ctx->cfg.sort_every > 1 && ctx->cfg.diag_every > 0)
        return fail(ctx, TG_ERR_ARG, "tg_shock_init: per-lap diagnostics with injection need sort_every = 1");
    if (k->dseed < 1.0 || k->dseed >= 2147483647.0 || k->dseed != floor(k->dseed))
        return fail(ctx, TG_ERR_ARG, "tg_shock_init: dseed must be an integer in [1, 2^31 - 2]");
    std::vector<float> tab(4 * (TG_PDF_SZ + 1));
    float *gti = tab.data(), *pti = gti + (TG_PDF_SZ + 1), *gte = pti + (TG_PDF_SZ + 1), *pte = gte + (TG_PDF_SZ + 1);
    maxw_table(k->delgam_i, ctx->g.dims, k->pcosthmult, gti, pti);
    maxw_table(k->delgam_e, ctx->g.dims, k->pcosthmult, gte, pte);
    if (!ctx->d_tables) {
        int r = dalloc(ctx, &ctx->d_tables, tab.size());
        if (!r) r = dalloc(ctx, &ctx->d_shock, 1);
        if (r) return r;
    }
    ShockParams K;
    memset(&K, 0, sizeof K);
    K.wall = k->wall;
    K.inject = k->inject;
    K.gammawall = k->gammawall;
    K.betawall = k->betawall;
    K.cond_i1 = k->cond_i1;
    K.cond_i2 = k->cond_i2;
    K.edge_i1 = k->edge_i1;
    K.edge_i2 = k->edge_i2;
    for (int a = 0; a < 6; a++) K.edge[a] = k->edge[a];
    K.xinj_max = k->xinj_max;
    K.ppc0 = k->ppc0;
    K.gamma_drift = k->gamma_drift;
    K.weight = k->weight;
    K.y1 = k->y1;
    K.y2 = k->y2;
    K.pcosthmult = k->pcosthmult;
    K.sigma_nonzero = k->sigma_nonzero;
    const size_t T = TG_PDF_SZ + 1;
    K.gt[0] = ctx->d_tables;
    K.pt[0] = ctx->d_tables + T;
    K.gt[1] = ctx->d_tables + 2 * T;
    K.pt[1] = ctx->d_tables + 3 * T;
    K.a13 = host_powmod31(16807, 13);
    if (K.cond_i1 != K.cond_i2 && (K.cond_i1 < 1 || K.cond_i2 > ctx->g.mx || K.cond_i1 > K.cond_i2))
        return fail(ctx, TG_ERR_ARG, "tg_shock_init: conductor columns outside [1, mx]");
    if (K.edge_i1 != K.edge_i2 && (K.edge_i1 < 1 || K.edge_i2 > ctx->g.mx || K.edge_i1 > K.edge_i2))
        return fail(ctx, TG_ERR_ARG, "tg_shock_init: edge columns outside [1, mx]");
    ShockState S;
    memset(&S, 0, sizeof S);
    S.xinject2 = k->xinject2;
    S.walloc = k->walloc;
    S.x2in = ctx->P.x2in;
    S.betainj = k->betainj;
    S.totalpartnum = k->totalpartnum;
    S.seed = (long long)k->dseed;
    S.weight = k->weight;
    CK(cudaMemcpyAsync(ctx->d_tables, tab.data(), tab.size() * 4, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaMemcpyAsync(ctx->d_shock, &S, sizeof S, cudaMemcpyHostToDevice, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    ctx->K = K;
    ctx->hshock = *k;
    ctx->shock_on = true;
    for (int p = 0; p < 2; p++)
        if (ctx->cycle[p]) {
            cudaGraphExecDestroy(ctx->cycle[p]);
            ctx->cycle[p] = nullptr;
        }
    return TG_OK;
}

extern "C" int tg_shock_get(tg_ctx *ctx, tg_shock *out) {
    if (!ctx || !out) return TG_ERR_ARG;
    if (!ctx->shock_on) return fail(ctx, TG_ERR_STATE, "tg_shock_get: hooks not set");
    ShockState S;
    CK(cudaMemcpyAsync(&S, ctx->d_shock, sizeof S, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    *out = ctx->hshock;
    out->xinject2 = S.xinject2;
    out->walloc = S.walloc;
    out->betainj = S.betainj;
    out->dseed = (double)S.seed;
    out->totalpartnum = S.totalpartnum;
    return check_status(ctx);
}

static const Species *cur_species(tg_ctx *ctx) { return ctx->sp[ctx->par]; }

// one injection: plan, a parallel pass over the pairs, finish; host-driven
// loads (lap = false) re-run the pass after a gamma redraw when many pairs
// follow it, so the finishing kernel's sequential tail stays short
static int inject_run(tg_ctx *ctx, int mode, float x1, float x2, float y1, float y2, float ppc, float weight,
                      bool in_lap, int *const *hist) {
    long long *cnt = ctx->d_cnt + 2 * ctx->par;
    CK(launch_inject_plan(ctx->g, ctx->P, ctx->K, ctx->d_shock, mode, x1, x2, y1, y2, ppc, weight, cnt,
                          ctx->cfg.maxhlf, ctx->d_status, ctx->st));
    CK(launch_inject_pairs(ctx->g, ctx->P, ctx->K, ctx->d_shock, cur_species(ctx), INJECT_GRID, ctx->d_status,
                           ctx->st));
    if (!in_lap) {
        for (;;) {
            ShockState S;
            CK(cudaMemcpyAsync(&S, ctx->d_shock, sizeof S, cudaMemcpyDeviceToHost, ctx->st));
            CK(cudaStreamSynchronize(ctx->st));
            if (S.first_redraw >= S.n || S.n - S.first_redraw <= 4096) break;
            CK(launch_inject_fixup(ctx->g, ctx->P, ctx->K, ctx->d_shock, ctx->st));
            CK(launch_inject_pairs(ctx->g, ctx->P, ctx->K, ctx->d_shock, cur_species(ctx), INJECT_GRID,
                                   ctx->d_status, ctx->st));
        }
    }
    CK(launch_inject_finish(ctx->g, ctx->P, ctx->K, ctx->d_shock, cur_species(ctx), cnt, hist, INJECT_GRID,
                            ctx->d_status, ctx->st));
    return TG_OK;
}

static int inject_lap(tg_ctx *ctx, bool sort_now) {
    return inject_run(ctx, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, true, sort_now ? ctx->hist : nullptr);
}

extern "C" int tg_inject_region(tg_ctx *ctx, float x1, float x2, float y1, float y2, float ppc, float weight) {
    if (!ctx) return TG_ERR_ARG;
    if (!ctx->shock_on) return fail(ctx, TG_ERR_STATE, "tg_inject_region: hooks not set (tg_shock_init)");
    if (!(x2 >= x1) || !(y2 >= y1)) return fail(ctx, TG_ERR_ARG, "tg_inject_region: x2 < x1 or y2 < y1");
    int r = inject_run(ctx, 1, x1, x2, y1, y2, ppc, weight, false, nullptr);
    if (r) return r;
    ctx->dirty = true;
    ctx->may_have_dead = true;
    return check_status(ctx);
}

extern "C" int tg_inject(tg_ctx *ctx) {
    if (!ctx) return TG_ERR_ARG;
    if (!ctx->shock_on) return fail(ctx, TG_ERR_STATE, "tg_inject: hooks not set (tg_shock_init)");
    int r = inject_run(ctx, 0, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, false, nullptr);
    if (r) return r;
    ctx->dirty = true;
    ctx->may_have_dead = true;
    return TG_OK;
}

extern "C" int tg_particle_bc(tg_ctx *ctx) {
    if (!ctx) return TG_ERR_ARG;
    if (!ctx->shock_on) return fail(ctx, TG_ERR_STATE, "tg_particle_bc: hooks not set (tg_shock_init)");
    float *cur3[3] = {ctx->f[6], ctx->f[7], ctx->f[8]};
    CK(launch_particle_bc(ctx->g, ctx->P, ctx->K, ctx->d_shock, cur_species(ctx), ctx->d_cnt + 2 * ctx->par,
                          count_hint(ctx, 0) + count_hint(ctx, 1), cur3, ctx->fix, ctx->d_status, ctx->d_dead,
                          ctx->st));
    ctx->may_have_dead = true;
    return TG_OK;
}

extern "C" int tg_field_bc(tg_ctx *ctx) {
    if (!ctx) return TG_ERR_ARG;
    if (!ctx->shock_on) return fail(ctx, TG_ERR_STATE, "tg_field_bc: hooks not set (tg_shock_init)");
    CK(launch_field_bc(ctx->g, ctx->K, ctx->f, ctx->st));
    return TG_OK;
}

// ---------------------------------------------------------------------------
// fused lap
// ---------------------------------------------------------------------------
static cudaError_t mark(tg_ctx *ctx, int li, int phase, int end) {
    if (!ctx->timing || li > ctx->ev_laps) return cudaSuccess;
    if (!end) ctx->ev_used[li][phase] = true;
    return cudaEventRecord(ctx->ev[((size_t)li * TG_NPHASES + phase) * 2 + end], ctx->st);
}

static int sort_species(tg_ctx *ctx, int s, bool counted);

static int lap_kernels(tg_ctx *ctx, bool sort_now, int *nk, int li = 0, const HostPipe *pipe = nullptr) {
    cudaStream_t st = ctx->st;
    const Geom &g = ctx->g;
    int k = 0;
    CK(mark(ctx, li, 0, 0));
    // bc_b1; bc_e1; advance_Bhalfstep; bc_b1  (tristanmainloop.F90:117-122)
    CK(launch_ghost(g, ctx->f[3], ctx->f[4], ctx->f[5], GHOST_BC, st)); k++;
    CK(launch_ghost(g, ctx->f[0], ctx->f[1], ctx->f[2], GHOST_BC, st)); k++;
    CK(launch_advance_b(g, ctx->P, ctx->f, st)); k++;
    CK(launch_ghost(g, ctx->f[3], ctx->f[4], ctx->f[5], GHOST_BC, st)); k++;
    if (g.dims == 3) { CK(launch_primal(g, ctx->f, ctx->prim, st)); k++; }
    // reset_currents (:175), then move_particles + deposit_particles fused
    // (:134, :183): the deposit reads no field and the field updates read
    // no current, so the current is deposited right after each push
    if (!ctx->P.fixed)
        for (int a = 6; a < 9; a++) CK(cudaMemsetAsync(ctx->f[a], 0, (size_t)g.lot * 4, st));
    CK(mark(ctx, li, 0, 1));
    CK(mark(ctx, li, 1, 0));
    if (pipe) {
        // part by part: the freshly uploaded records into the particle
        // arrays, the part's tile sort (into the other parity), its push, and
        // its records back to the staging copy, from where they go home
        const int p0 = ctx->par;
        CK(cudaMemsetAsync(ctx->d_dead, 0, sizeof(int), st));  // the sorts compact
        ctx->fault_seen = false;
        for (int s = 0; s < 2; s++) {
            const size_t soff = s == 0 ? 0 : (size_t)ctx->cfg.maxhlf * AOS;
            // a record dropped on the way up leaves its part one entry short:
            // the entries no sort fills read as dropped
            if (pipe->parts > 1)
                CK(cudaMemsetAsync(ctx->sp[1 - p0][s].cell, 0xff, (size_t)ctx->host_n[s] * 4, st));
            for (int h = 0; h < pipe->parts; h++) {
                const long long o = pipe->off[s][h], m = pipe->off[s][h + 1] - o;
                const Species src = species_at(ctx->sp[p0][s], o), dst = species_at(ctx->sp[1 - p0][s], o);
                char *stg = pipe->stage + soff + (size_t)o * AOS;
                // the part's record count in, its sorted count out
                long long *cin = ctx->d_cnt + 2 * p0 + s, *cout = ctx->d_cnt + 2 * (1 - p0) + s;
                if (pipe->parts > 1) {
                    cin = ctx->d_pcnt + 2 * (s * TG_HOST_PARTS_MAX + h);
                    cout = cin + 1;
                }
                CK(cudaStreamWaitEvent(st, pipe->uploaded[s][h], 0));
                CK(launch_aos_to_soa(g, stg, src, m, ctx->d_status, st));
                CK(launch_tile_count(g, src, cin, m, ctx->hist[s], st));
                int *ts = pipe->ts[s][h];
                CK(launch_scan(ctx->hist[s], ts, ctx->cursor[s], g.ntiles, cout, st));
                CK(launch_scatter(g, src, dst, cin, m, ts, ctx->cursor[s], st));
                TileArgs a = tile_args(ctx, false);
                a.sp[s] = dst;
                a.tstart[s] = ts;
                a.only = s + 1;
                CK(launch_tiles(a, ctx->P.fixed != 0, true, true, st));
                CK(launch_soa_to_aos(g, dst, stg, m, st));
                CK(cudaEventRecord(pipe->pushed[s][h], st));
                CK(cudaStreamWaitEvent(pipe->down, pipe->pushed[s][h], 0));
                CK(cudaMemcpyAsync(pipe->host + soff + (size_t)o * AOS, stg, (size_t)m * AOS,
                                   cudaMemcpyDeviceToHost, pipe->down));
                k += 6;
                if (ctx->cfg.diag_every > 0) {
                    // the part's share of the diagnostics' particle pass, while
                    // the part goes home and later parts arrive
                    DiagLaunch d = diag_launch(ctx);
                    d.sp[s] = dst;
                    d.tstart[s] = ts;
                    d.only = s + 1;
                    CK(launch_diag_particles(d, st));
                    k++;
                }
            }
        }
        ctx->par = 1 - p0;
        // in parts the species is grouped by tile part by part only
        ctx->dirty = pipe->parts > 1;
        ctx->may_have_dead = false;
    }
    TileArgs a = tile_args(ctx, sort_now);
    // particle_bc_user (the wall) runs inside the tile kernel, between the
    // push and the deposit; the wall advances first
    if (ctx->shock_on && ctx->K.wall) { CK(launch_wall_step(ctx->P, ctx->K, ctx->d_shock, st)); k++; }
    if (!pipe) { CK(launch_tiles(a, ctx->P.fixed != 0, true, true, st)); k++; }
    if (ctx->shock_on && ctx->cfg.sort_every > 1) {
        // the particles injected since the last sort
        CK(launch_tail(a, ctx->d_cnt + 2 * ctx->par, ctx->P.fixed != 0, st)); k++;
    }
    CK(mark(ctx, li, 1, 1));
    CK(mark(ctx, li, 2, 0));
    // advance_Bhalfstep; bc_b1; bc_b2 (:139-145); [field_bc_user];
    // advance_Efield; [field_bc_user]; bc_e2; [field_bc_user]
    CK(launch_advance_b(g, ctx->P, ctx->f, st)); k++;
    CK(launch_ghost(g, ctx->f[3], ctx->f[4], ctx->f[5], GHOST_BC, st)); k++;
    if (ctx->shock_on) { CK(launch_field_bc(g, ctx->K, ctx->f, st)); k++; }
    CK(launch_advance_e(g, ctx->P, ctx->f, st)); k++;
    if (ctx->shock_on) { CK(launch_field_bc(g, ctx->K, ctx->f, st)); k++; }
    CK(launch_ghost(g, ctx->f[0], ctx->f[1], ctx->f[2], GHOST_BC, st)); k++;
    if (ctx->shock_on) { CK(launch_field_bc(g, ctx->K, ctx->f, st)); k++; }
    CK(mark(ctx, li, 2, 1));
    CK(mark(ctx, li, 3, 0));
    if (ctx->P.fixed) {
        float *cur3[3] = {ctx->f[6], ctx->f[7], ctx->f[8]};
        CK(launch_fixed_to_float(g, ctx->P, ctx->fix, cur3, st)); k++;
    }
    // exchange_current; apply_filter1_opt; add_current (:201-242)
    CK(launch_fold(g, ctx->P, ctx->f + 6, st)); k += fold_launches(g);
    CK(mark(ctx, li, 3, 1));
    CK(mark(ctx, li, 4, 0));
    int r = filter_passes(ctx);
    if (r) return r;
    k += ctx->cfg.ntimes;
    CK(mark(ctx, li, 4, 1));
    CK(mark(ctx, li, 5, 0));
    CK(launch_add_current(g, ctx->f, st)); k++;
    if (ctx->shock_on) {
        // field_bc_user; inject_particles_user (:242-262); the injected
        // particles join the tile histogram of this lap's sort
        CK(launch_field_bc(g, ctx->K, ctx->f, st)); k++;
        int rr = inject_lap(ctx, sort_now);
        if (rr) return rr;
        k += 4;
    }
    CK(mark(ctx, li, 5, 1));
    if (pipe) {
        // the fields are final here (the diagnostics only read them): they
        // go home while the diagnostics run
        CK(cudaEventRecord(ctx->ev_link[0], st));
        CK(cudaStreamWaitEvent(pipe->down, ctx->ev_link[0], 0));
        for (int f9 = 0; f9 < 9; f9++)
            CK(cudaMemcpyAsync(ctx->hf[f9], ctx->f[f9], (size_t)g.lot * 4, cudaMemcpyDeviceToHost, pipe->down));
    }
    if (sort_now && !pipe) {
        CK(mark(ctx, li, 6, 0));
        int rr = sort_all(ctx, true);
        if (rr) return rr;
        k += 4;
        CK(mark(ctx, li, 6, 1));
    }
    if (ctx->cfg.diag_every > 0) {
        CK(mark(ctx, li, 7, 0));
        int rr = run_diag(ctx, !pipe);
        if (rr) return rr;
        k += 3 + ctx->cfg.ntimes + (pipe ? 0 : 1);
        CK(mark(ctx, li, 7, 1));
    }
    *nk = k;
    return TG_OK;
}

static int capture_cycle(tg_ctx *ctx, int start_par) {
    const int se = ctx->cfg.sort_every < 1 ? 1 : ctx->cfg.sort_every;
    cudaGraph_t graph = nullptr;
    CK(cudaStreamBeginCapture(ctx->st, cudaStreamCaptureModeThreadLocal));
    int r = TG_OK, nk = 0;
    for (int l = 0; l < 2 * se && r == TG_OK; l++)
        r = lap_kernels(ctx, (l % se) == se - 1, &nk, l < ctx->ev_laps ? l : 1 << 20);
    cudaError_t e = cudaStreamEndCapture(ctx->st, &graph);
    if (r) {
        if (graph) cudaGraphDestroy(graph);
        return r;
    }
    if (e != cudaSuccess) return fail(ctx, TG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&ctx->cycle[start_par], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return fail(ctx, TG_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    ctx->kernels_per_step = nk;
    // capturing walked the parity through two sorts: back where it started
    ctx->par = start_par;
    return TG_OK;
}

extern "C" int tg_step(tg_ctx *ctx, int32_t nsteps) {
    TG_RANGE("tg_step (main loop laps)");
    if (!ctx || nsteps < 0) return TG_ERR_ARG;
    int r = ensure_sorted(ctx);
    if (r) return r;
    if (nsteps > 0) ctx->may_have_dead = true;
    const int se = ctx->cfg.sort_every < 1 ? 1 : ctx->cfg.sort_every;
    const int cyc = 2 * se;
    int left = nsteps;
    // laps are replayed in whole sort cycles from a graph; the phase within a
    // cycle is tracked by the lap counter
    while (left > 0) {
        const int phase = (int)(ctx->lap % cyc);
        // with timing on, the last lap always runs outside the graph: CUDA
        // events recorded by graph nodes cannot be read back for elapsed time
        const bool keep_last_direct = ctx->timing && left == cyc;
        if (phase == 0 && left >= cyc && !keep_last_direct) {
            const int p = ctx->par;
            if (!ctx->cycle[p]) {
                if ((r = capture_cycle(ctx, p))) return r;
            }
            CK(cudaGraphLaunch(ctx->cycle[p], ctx->st));
            // two sorts per cycle: parity unchanged
            ctx->lap += cyc;
            left -= cyc;
            ctx->last_laps = cyc;
            ctx->last_direct = false;
        } else {
            int nk = 0;
            // laps outside the graph time into their own event row
            if ((r = lap_kernels(ctx, (phase % se) == se - 1, &nk, ctx->ev_laps))) return r;
            ctx->last_laps = 1;
            ctx->last_direct = true;
            ctx->kernels_per_step = nk;
            ctx->lap += 1;
            left -= 1;
        }
    }
    return TG_OK;
}

extern "C" int tg_step_timed(tg_ctx *ctx, int32_t nsteps, float *ms) {
    if (!ctx || !ms) return TG_ERR_ARG;
    int r = ensure_sorted(ctx);
    if (r) return r;
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, ctx->st));
    r = tg_step(ctx, nsteps);
    CK(cudaEventRecord(b, ctx->st));
    CK(cudaEventSynchronize(b));
    CK(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (r) return r;
    return check_status(ctx);
}

// One main-loop pass with the bound host arrays as the state: E, B and the
// particle records go up, the lap runs, every field and record comes back.
// With page-locked host records on an all-periodic domain (no particle can
// leave) the transfers overlap the lap species by species; otherwise the
// same steps run one after another.
static int host_lap(tg_ctx *ctx) {
    const Geom &g = ctx->g;
    const bool periodic = g.per[0] && g.per[1] && (g.dims == 2 || g.per[2]);
    bool bound = ctx->hp != nullptr;
    for (int a = 0; a < 9; a++) bound = bound && ctx->hf[a] != nullptr;
    // page-locked records (the copies are then asynchronous DMA)
    const bool locked = bound && host_view(ctx, ctx->hp) != nullptr;
    if (!(locked && periodic && !ctx->shock_on)) {
        int r = tg_sync_from_host(ctx, TG_SYNC_E | TG_SYNC_B | TG_SYNC_PARTICLES);
        if (!r) r = tg_step(ctx, 1);
        if (!r) r = tg_sync_to_host(ctx, TG_SYNC_ALL);
        return r;
    }
    const long long n[2] = {*ctx->hions, *ctx->hlecs};
    for (int s = 0; s < 2; s++)
        if (n[s] < 0 || n[s] > ctx->cfg.maxhlf)
            return fail(ctx, TG_ERR_OVERFLOW, "species %d count %lld outside [0, maxhlf=%lld]", s, n[s],
                        (long long)ctx->cfg.maxhlf);
    if (!ctx->st_up) {
        CK(cudaStreamCreateWithFlags(&ctx->st_up, cudaStreamNonBlocking));
        CK(cudaStreamCreateWithFlags(&ctx->st_down, cudaStreamNonBlocking));
        for (auto &e : ctx->ev_link) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (!ctx->stage2) CK(cudaMalloc(&ctx->stage2, (size_t)ctx->cfg.maxhlf * AOS * 2 + 256));
    HostPipe pipe;
    pipe.host = (char *)ctx->hp;
    pipe.stage = (char *)ctx->stage2;
    pipe.down = ctx->st_down;
    cudaStream_t st = ctx->st;
    const size_t lot = (size_t)g.lot;
    CK(cudaStreamSynchronize(st));
    // parts per species: as set, else about 512 records of the larger
    // species per tile and part (measured best on the 2D and 3D benchmark
    // plasmas: every part's tile launch clears and flushes every tile's
    // window, so smaller parts pay that per-tile cost more often, larger
    // ones overlap less of the transfers)
    int parts = ctx->host_parts;
    if (parts == 0) {
        const long long big = n[0] > n[1] ? n[0] : n[1];
        parts = (int)((big + 256LL * g.ntiles) / (512LL * g.ntiles));
        parts = parts < 1 ? 1 : parts > TG_HOST_PARTS_MAX ? TG_HOST_PARTS_MAX : parts;
    }
    pipe.parts = parts;
    if (parts > 1 && !ctx->d_pcnt) {
        int rr = dalloc(ctx, &ctx->d_pcnt, (size_t)4 * TG_HOST_PARTS_MAX);
        for (int s = 0; s < 2 && !rr; s++)
            for (int h = 1; h < TG_HOST_PARTS_MAX && !rr; h++)
                rr = dalloc(ctx, &ctx->ptstart[s][h], (size_t)g.ntiles + 1);
        if (rr) return rr;
    }
    // the first part of the first species and the last part of the second
    // get a third of the others' share: only one direction of the link is
    // busy while the first part goes up and while the last one comes home
    long long cum[2][TG_HOST_PARTS_MAX + 1];
    for (int s = 0; s < 2; s++) {
        cum[s][0] = 0;
        for (int h = 0; h < parts; h++)
            cum[s][h + 1] = cum[s][h] + ((parts > 1 && h == (s == 0 ? 0 : parts - 1)) ? 1 : 3);
    }
    for (int s = 0; s < 2; s++) {
        for (int h = 0; h <= parts; h++) {
            // part boundaries on multiples of 32 records (whole 128-byte lines of the arrays)
            pipe.off[s][h] = h == parts ? n[s] : (n[s] * cum[s][h] / cum[s][parts]) & ~31LL;
            if (h < parts) {
                pipe.ts[s][h] = h == 0 ? ctx->tstart[s] : ctx->ptstart[s][h];
                pipe.uploaded[s][h] = ctx->ev_link[1 + 2 * (s * TG_HOST_PARTS_MAX + h)];
                pipe.pushed[s][h] = ctx->ev_link[2 + 2 * (s * TG_HOST_PARTS_MAX + h)];
            }
        }
        for (int h = 0; h < parts; h++) ctx->pcnt[s][h][0] = pipe.off[s][h + 1] - pipe.off[s][h];
    }
    for (int s = 0; s < 2; s++) {
        ctx->host_n[s] = n[s];
        ctx->hcount[s] = n[s];
        CK(cudaMemcpyAsync(ctx->d_cnt + 2 * ctx->par + s, &ctx->host_n[s], sizeof(long long),
                           cudaMemcpyHostToDevice, st));
        // in parts the counts of the lap's parity are the whole species'
        if (parts > 1)
            CK(cudaMemcpyAsync(ctx->d_cnt + 2 * (1 - ctx->par) + s, &ctx->host_n[s], sizeof(long long),
                               cudaMemcpyHostToDevice, st));
    }
    if (parts > 1)
        CK(cudaMemcpyAsync(ctx->d_pcnt, ctx->pcnt, sizeof ctx->pcnt, cudaMemcpyHostToDevice, st));
    // E and B first: host-to-device copies leave in the order they are
    // issued, and the lap's first phases need the fields only
    for (int a = 0; a < 6; a++) CK(cudaMemcpyAsync(ctx->f[a], ctx->hf[a], lot * 4, cudaMemcpyHostToDevice, st));
    // the records go up by DMA once earlier work on the stream is done
    CK(cudaEventRecord(ctx->ev_link[0], st));
    CK(cudaStreamWaitEvent(ctx->st_up, ctx->ev_link[0], 0));
    for (int s = 0; s < 2; s++) {
        const size_t soff = s == 0 ? 0 : (size_t)ctx->cfg.maxhlf * AOS;
        for (int h = 0; h < parts; h++) {
            const size_t o = soff + (size_t)pipe.off[s][h] * AOS;
            CK(cudaMemcpyAsync(pipe.stage + o, pipe.host + o, (size_t)(pipe.off[s][h + 1] - pipe.off[s][h]) * AOS,
                               cudaMemcpyHostToDevice, ctx->st_up));
            CK(cudaEventRecord(pipe.uploaded[s][h], ctx->st_up));
        }
    }
    int nk = 0;
    int r = lap_kernels(ctx, false, &nk, 1 << 20, &pipe);
    if (r) return r;
    ctx->kernels_per_step = nk;
    ctx->last_laps = 1;
    ctx->last_direct = true;
    ctx->lap += 1;
    CK(cudaEventRecord(ctx->ev_link[0], ctx->st_down));
    CK(cudaStreamWaitEvent(st, ctx->ev_link[0], 0));
    int flags[2] = {0, 0};
    CK(cudaMemcpyAsync(&flags[0], ctx->d_dead, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&flags[1], ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (flags[0] || flags[1]) {
        // a record was dropped (outside the grid on the way up, or a fault):
        // send the compacted records instead, and report the fault
        ctx->may_have_dead = true;
        return tg_sync_to_host(ctx, TG_SYNC_PARTICLES);
    }
    *ctx->hions = (int32_t)n[0];
    *ctx->hlecs = (int32_t)n[1];
    return TG_OK;
}

extern "C" int tg_set_host_parts(tg_ctx *ctx, int32_t parts) {
    if (!ctx) return TG_ERR_ARG;
    if (parts < 0 || parts > TG_HOST_PARTS_MAX)
        return fail(ctx, TG_ERR_ARG, "tg_set_host_parts: parts %d outside [0, %d]", parts, TG_HOST_PARTS_MAX);
    ctx->host_parts = parts;
    return TG_OK;
}

#ifndef MADV_COLLAPSE
#define MADV_COLLAPSE 25  // Linux 6.1+: back the populated range with huge pages now
#endif
// Ask for transparent huge pages behind a host range before it is
// page-locked: page-locked base pages sustain fewer bytes per second over
// the host link when both directions are in flight. Advice only: a kernel
// or mapping that refuses it leaves the range as it was.
static void advise_huge_pages(void *h, size_t len) {
    const long ps = sysconf(_SC_PAGESIZE);
    if (ps <= 0) return;
    const uintptr_t a = ((uintptr_t)h + (uintptr_t)ps - 1) & ~((uintptr_t)ps - 1);
    const uintptr_t b = ((uintptr_t)h + len) & ~((uintptr_t)ps - 1);
    if (b <= a) return;
    (void)madvise((void *)a, b - a, MADV_HUGEPAGE);
    (void)madvise((void *)a, b - a, MADV_COLLAPSE);
}

extern "C" int tg_pin_host(tg_ctx *ctx) {
    if (!ctx) return TG_ERR_ARG;
    if (!ctx->hp) return fail(ctx, TG_ERR_STATE, "tg_pin_host: particles not bound");
    void *h[10];
    size_t len[10];
    int n = 0;
    for (int a = 0; a < 9; a++)
        if (ctx->hf[a]) {
            h[n] = ctx->hf[a];
            len[n++] = (size_t)ctx->g.lot * 4;
        }
    h[n] = ctx->hp;
    len[n++] = (size_t)ctx->cfg.maxhlf * AOS * 2;
    for (int i = 0; i < n; i++) {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, h[i]) == cudaSuccess && at.type == cudaMemoryTypeHost) continue;
        (void)cudaGetLastError();
        advise_huge_pages(h[i], len[i]);
        cudaError_t e = cudaHostRegister(h[i], len[i], cudaHostRegisterDefault);
        if (e == cudaErrorHostMemoryAlreadyRegistered) {
            (void)cudaGetLastError();
            continue;
        }
        if (e != cudaSuccess) return fail(ctx, TG_ERR_CUDA, "tg_pin_host: cudaHostRegister: %s", cudaGetErrorString(e));
        ctx->pinned.push_back(h[i]);
    }
    return TG_OK;
}

extern "C" int tg_step_host(tg_ctx *ctx, int32_t nsteps) {
    TG_RANGE("tg_step_host (main loop laps, host state)");
    if (!ctx || nsteps < 0) return TG_ERR_ARG;
    for (int l = 0; l < nsteps; l++) {
        int r = host_lap(ctx);
        if (r) return r;
    }
    return TG_OK;
}

extern "C" int tg_enable_timing(tg_ctx *ctx, int32_t on) {
    if (!ctx) return TG_ERR_ARG;
    CK(cudaStreamSynchronize(ctx->st));
    for (int p = 0; p < 2; p++)
        if (ctx->cycle[p]) {
            cudaGraphExecDestroy(ctx->cycle[p]);
            ctx->cycle[p] = nullptr;
        }
    if (on && ctx->ev.empty()) {
        const int se = ctx->cfg.sort_every < 1 ? 1 : ctx->cfg.sort_every;
        ctx->ev_laps = 2 * se < 64 ? 2 * se : 64;
        ctx->ev.resize((size_t)(ctx->ev_laps + 1) * TG_NPHASES * 2);
        for (auto &e : ctx->ev) CK(cudaEventCreate(&e));
    }
    ctx->timing = on != 0;
    memset(ctx->ev_used, 0, sizeof ctx->ev_used);
    return TG_OK;
}

extern "C" int tg_phase_times(tg_ctx *ctx, float *ms, int32_t nphases) {
    if (!ctx || !ms) return TG_ERR_ARG;
    if (!ctx->timing) return fail(ctx, TG_ERR_STATE, "tg_phase_times: timing not enabled");
    CK(cudaStreamSynchronize(ctx->st));
    const int laps = ctx->last_direct ? 1 : (ctx->last_laps < ctx->ev_laps ? ctx->last_laps : ctx->ev_laps);
    const int row0 = ctx->last_direct ? ctx->ev_laps : 0;
    for (int ph = 0; ph < nphases && ph < TG_NPHASES; ph++) {
        float sum = 0.0f;
        for (int li = row0; li < row0 + laps; li++) {
            if (!ctx->ev_used[li][ph]) continue;
            float t = 0.0f;
            const size_t b = ((size_t)li * TG_NPHASES + ph) * 2;
            if (cudaEventElapsedTime(&t, ctx->ev[b], ctx->ev[b + 1]) != cudaSuccess) {
                (void)cudaGetLastError();
                sum = -1.0f;  // event pair not timed
                break;
            }
            sum += t;
        }
        ms[ph] = (laps > 0 && sum >= 0.0f) ? sum / (float)laps : -1.0f;
    }
    return TG_OK;
}

extern "C" int tg_diag_fp64(tg_ctx *ctx, tg_diag *out) {
    TG_RANGE("tg_diag_fp64");
    if (!ctx || !out) return TG_ERR_ARG;
    // injected particles may sit past the tile ranges since the last sort
    if (ctx->shock_on && ctx->cfg.sort_every > 1) ctx->dirty = true;
    int r = ensure_sorted(ctx);
    if (r) return r;
    if ((r = run_diag(ctx, true))) return r;
    double h[16];
    if (tg_diag_history(ctx, h, 1) != 1) return fail(ctx, TG_ERR_STATE, "tg_diag_fp64: no record");
    record_to_diag(h, out);
    return check_status(ctx);
}

// ---------------------------------------------------------------------------
// restart files in the reference's format (write_restart,
// code/output.F90:2192-2222; restart, code/restart.F90:209-255): one
// gfortran unformatted sequential record per file, split into subrecords of
// at most 2147483639 bytes whose signed 4-byte markers say whether the
// record continues (leading marker < 0) or continues a previous subrecord
// (trailing marker < 0)
// ---------------------------------------------------------------------------
namespace {
const int64_t GFORTRAN_MAX_SUBRECORD = 2147483639LL;

struct RecordWriter {
    FILE *f = nullptr;
    int64_t max_sub = GFORTRAN_MAX_SUBRECORD;
    int64_t total = 0, written = 0, in_sub = 0, sub_len = 0;
    bool first = true, ok = true;
    void marker(int32_t m) { ok = ok && fwrite(&m, 4, 1, f) == 1; }
    void open_sub() {
        sub_len = std::min(max_sub, total - written);
        const bool last = written + sub_len >= total;
        marker(last ? (int32_t)sub_len : -(int32_t)sub_len);
        in_sub = 0;
    }
    void close_sub() {
        marker(first ? (int32_t)sub_len : -(int32_t)sub_len);
        first = false;
    }
    void begin(int64_t bytes) {
        total = bytes;
        written = 0;
        first = true;
        open_sub();
        if (total == 0) close_sub();
    }
    void put(const void *p, int64_t n) {
        const unsigned char *c = (const unsigned char *)p;
        while (n > 0 && ok) {
            const int64_t k = std::min(n, sub_len - in_sub);
            ok = ok && fwrite(c, 1, (size_t)k, f) == (size_t)k;
            c += k;
            n -= k;
            in_sub += k;
            written += k;
            if (in_sub == sub_len) {
                close_sub();
                if (written < total) open_sub();
            }
        }
    }
};

// one whole logical record
bool read_record(FILE *f, std::vector<unsigned char> &out) {
    out.clear();
    bool first = true;
    for (;;) {
        int32_t lead = 0, tail = 0;
        if (fread(&lead, 4, 1, f) != 1) return false;
        const int64_t len = lead < 0 ? -(int64_t)lead : lead;
        const size_t at = out.size();
        out.resize(at + (size_t)len);
        if (len > 0 && fread(out.data() + at, 1, (size_t)len, f) != (size_t)len) return false;
        if (fread(&tail, 4, 1, f) != 1) return false;
        const int64_t tlen = tail < 0 ? -(int64_t)tail : tail;
        if (tlen != len || (tail < 0) == first) return false;
        first = false;
        if (lead >= 0) return true;
    }
}

struct Cursor {
    const unsigned char *p, *end;
    template <class T>
    bool get(T &v) {
        if (end - p < (ptrdiff_t)sizeof(T)) return false;
        memcpy(&v, p, sizeof(T));
        p += sizeof(T);
        return true;
    }
    bool take(void *dst, size_t n) {
        if ((size_t)(end - p) < n) return false;
        memcpy(dst, p, n);
        p += n;
        return true;
    }
};

struct AosRec {
    float x, y, z, u, v, w, ch;
    int32_t ind, proc, splitlev;
};
}  // namespace

extern "C" int tg_write_restart(tg_ctx *ctx, const char *fld_path, const char *prt_path,
                                const tg_restart_meta *meta) {
    if (!ctx || !fld_path || !prt_path || !meta) return TG_ERR_ARG;
    tg_restart_meta m = *meta;
    if (ctx->shock_on) {
        ShockState S;
        CK(cudaMemcpyAsync(&S, ctx->d_shock, sizeof S, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        m.dseed = (double)S.seed;
        m.xinject2 = S.xinject2;
        m.walloc = S.walloc;
        m.totalpartnum = S.totalpartnum;
    }
    const int64_t max_sub = m.max_subrecord > 0 ? m.max_subrecord : GFORTRAN_MAX_SUBRECORD;
    const size_t lot = (size_t)ctx->g.lot;
    // fields
    std::vector<float> fl(6 * lot);
    for (int a = 0; a < 6; a++)
        CK(cudaMemcpyAsync(fl.data() + a * lot, ctx->f[a], lot * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    FILE *f = fopen(fld_path, "wb");
    if (!f) return fail(ctx, TG_ERR_ARG, "tg_write_restart: cannot open %s", fld_path);
    RecordWriter w;
    w.f = f;
    w.max_sub = max_sub;
    const int32_t dims3[3] = {ctx->g.mx, ctx->g.my, ctx->g.mz};
    w.begin(12 + 24 * (int64_t)lot + 8 + 4 + 24 + 4 + 8);
    w.put(dims3, 12);
    w.put(fl.data(), 24 * (int64_t)lot);
    w.put(&m.dseed, 8);
    w.put(&m.lap, 4);
    w.put(&m.xinject, 8);
    w.put(&m.xinject2, 8);
    w.put(&m.xinject3, 8);
    w.put(&m.leftwall, 4);
    w.put(&m.walloc, 8);
    const bool okf = w.ok && fclose(f) == 0;
    if (!okf) return fail(ctx, TG_ERR_ARG, "tg_write_restart: write to %s failed", fld_path);
    // particles
    long long n[2];
    int r = exact_counts(ctx, n);
    if (r) return r;
    if (!ctx->stage) CK(cudaMalloc(&ctx->stage, (size_t)ctx->cfg.maxhlf * AOS + 256));
    std::vector<AosRec> pa[2];
    for (int s = 0; s < 2; s++) {
        pa[s].resize((size_t)n[s]);
        if (n[s] == 0) continue;
        CK(launch_soa_to_aos(ctx->g, ctx->sp[ctx->par][s], ctx->stage, n[s], ctx->st));
        CK(cudaMemcpyAsync(pa[s].data(), ctx->stage, (size_t)n[s] * AOS, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
    }
    f = fopen(prt_path, "wb");
    if (!f) return fail(ctx, TG_ERR_ARG, "tg_write_restart: cannot open %s", prt_path);
    RecordWriter wp;
    wp.f = f;
    wp.max_sub = max_sub;
    const int32_t head[5] = {(int32_t)n[0], (int32_t)n[1], m.maxptl > 0 ? m.maxptl : (int32_t)(2 * ctx->cfg.maxhlf),
                             (int32_t)ctx->cfg.maxhlf, m.totalpartnum};
    wp.begin(20 + 40 * (n[0] + n[1]));
    wp.put(head, 20);
    std::vector<char> col;
    for (int comp = 0; comp < 10; comp++)
        for (int s = 0; s < 2; s++) {
            col.resize((size_t)n[s] * 4);
            for (long long i = 0; i < n[s]; i++)
                memcpy(col.data() + 4 * i, (const char *)&pa[s][(size_t)i] + 4 * comp, 4);
            wp.put(col.data(), (int64_t)col.size());
        }
    const bool okp = wp.ok && fclose(f) == 0;
    if (!okp) return fail(ctx, TG_ERR_ARG, "tg_write_restart: write to %s failed", prt_path);
    return check_status(ctx);
}

extern "C" int tg_read_restart(tg_ctx *ctx, const char *fld_path, const char *prt_path, tg_restart_meta *out) {
    if (!ctx || !fld_path || !prt_path || !out) return TG_ERR_ARG;
    std::vector<unsigned char> rec;
    FILE *f = fopen(fld_path, "rb");
    if (!f) return fail(ctx, TG_ERR_ARG, "tg_read_restart: cannot open %s", fld_path);
    const bool okr = read_record(f, rec);
    fclose(f);
    if (!okr) return fail(ctx, TG_ERR_ARG, "tg_read_restart: %s is not one unformatted record", fld_path);
    const size_t lot = (size_t)ctx->g.lot;
    Cursor c{rec.data(), rec.data() + rec.size()};
    int32_t d3[3];
    if (!c.take(d3, 12) || d3[0] != ctx->g.mx || d3[1] != ctx->g.my || d3[2] != ctx->g.mz)
        return fail(ctx, TG_ERR_ARG, "tg_read_restart: grid %d x %d x %d does not match the context", d3[0], d3[1],
                    d3[2]);
    std::vector<float> fl(6 * lot);
    tg_restart_meta m;
    memset(&m, 0, sizeof m);
    if (!c.take(fl.data(), 24 * lot) || !c.get(m.dseed) || !c.get(m.lap) || !c.get(m.xinject) ||
        !c.get(m.xinject2) || !c.get(m.xinject3) || !c.get(m.leftwall) || !c.get(m.walloc))
        return fail(ctx, TG_ERR_ARG, "tg_read_restart: %s is short", fld_path);
    f = fopen(prt_path, "rb");
    if (!f) return fail(ctx, TG_ERR_ARG, "tg_read_restart: cannot open %s", prt_path);
    const bool okp = read_record(f, rec);
    fclose(f);
    if (!okp) return fail(ctx, TG_ERR_ARG, "tg_read_restart: %s is not one unformatted record", prt_path);
    Cursor p{rec.data(), rec.data() + rec.size()};
    int32_t head[5];
    if (!p.take(head, 20)) return fail(ctx, TG_ERR_ARG, "tg_read_restart: %s is short", prt_path);
    const long long n[2] = {head[0], head[1]};
    for (int s = 0; s < 2; s++)
        if (n[s] < 0 || n[s] > ctx->cfg.maxhlf)
            return fail(ctx, TG_ERR_OVERFLOW, "tg_read_restart: species %d count %lld outside [0, maxhlf=%lld]", s,
                        n[s], (long long)ctx->cfg.maxhlf);
    if ((size_t)(p.end - p.p) < (size_t)(40 * (n[0] + n[1])))
        return fail(ctx, TG_ERR_ARG, "tg_read_restart: %s is short", prt_path);
    m.maxptl = head[2];
    m.totalpartnum = head[4];
    std::vector<AosRec> pa[2];
    for (int s = 0; s < 2; s++) pa[s].resize((size_t)n[s]);
    for (int comp = 0; comp < 10; comp++)
        for (int s = 0; s < 2; s++)
            for (long long i = 0; i < n[s]; i++) {
                memcpy((char *)&pa[s][(size_t)i] + 4 * comp, p.p, 4);
                p.p += 4;
            }
    // upload
    for (int a = 0; a < 6; a++)
        CK(cudaMemcpyAsync(ctx->f[a], fl.data() + a * lot, lot * 4, cudaMemcpyHostToDevice, ctx->st));
    if (!ctx->stage) CK(cudaMalloc(&ctx->stage, (size_t)ctx->cfg.maxhlf * AOS + 256));
    for (int s = 0; s < 2; s++) {
        if (n[s] > 0) {
            CK(cudaMemcpyAsync(ctx->stage, pa[s].data(), (size_t)n[s] * AOS, cudaMemcpyHostToDevice, ctx->st));
            CK(launch_aos_to_soa(ctx->g, ctx->stage, ctx->sp[ctx->par][s], n[s], ctx->d_status, ctx->st));
        }
        CK(cudaMemcpyAsync(ctx->d_cnt + 2 * ctx->par + s, &n[s], sizeof(long long), cudaMemcpyHostToDevice,
                           ctx->st));
        ctx->hcount[s] = n[s];
    }
    if (ctx->shock_on) {
        ShockState S;
        CK(cudaMemcpyAsync(&S, ctx->d_shock, sizeof S, cudaMemcpyDeviceToHost, ctx->st));
        CK(cudaStreamSynchronize(ctx->st));
        S.seed = (long long)m.dseed;
        S.xinject2 = m.xinject2;
        S.walloc = m.walloc;
        S.totalpartnum = m.totalpartnum;
        if (ctx->K.inject) S.x2in = m.xinject2;
        CK(cudaMemcpyAsync(ctx->d_shock, &S, sizeof S, cudaMemcpyHostToDevice, ctx->st));
    }
    CK(cudaStreamSynchronize(ctx->st));  // host vectors live on this frame
    ctx->dirty = true;
    ctx->may_have_dead = true;
    *out = m;
    return check_status(ctx);
}

// ---------------------------------------------------------------------------
// grid moments for output (meanq_fld_cur, code/output.F90:5222-5482)
// ---------------------------------------------------------------------------
extern "C" int tg_moments(tg_ctx *ctx, int32_t kind, int32_t idx, int32_t idy, int32_t idz, float *num,
                          float *den) {
    if (!ctx || !num || !den) return TG_ERR_ARG;
    if (kind < 0 || kind >= TG_MOMENT_KINDS) return fail(ctx, TG_ERR_ARG, "tg_moments: kind %d unknown", kind);
    if (idx < 0 || idy < 0 || idz < 0) return fail(ctx, TG_ERR_ARG, "tg_moments: negative box half-width");
    const size_t lot = (size_t)ctx->g.lot;
    if (!ctx->mom[0]) {
        int r = dalloc(ctx, &ctx->mom[0], lot);
        if (!r) r = dalloc(ctx, &ctx->mom[1], lot);
        if (r) return r;
        CK(cudaMemsetAsync(ctx->mom[0], 0, lot * 8, ctx->st));
        CK(cudaMemsetAsync(ctx->mom[1], 0, lot * 8, ctx->st));
    }
    long long n[2];
    int r = exact_counts(ctx, n);
    if (r) return r;
    float *f3[3] = {ctx->ftmp[0], ctx->ftmp[1], ctx->ftmp[2]};
    CK(launch_moments(ctx->g, ctx->P, ctx->sp[ctx->par], ctx->d_cnt + 2 * ctx->par, n[0] + n[1], kind, idx, idy,
                      ctx->g.dims == 3 ? idz : 0, ctx->mom[0], ctx->mom[1], f3, ctx->st));
    CK(cudaMemcpyAsync(num, f3[0], lot * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaMemcpyAsync(den, f3[1], lot * 4, cudaMemcpyDeviceToHost, ctx->st));
    CK(cudaStreamSynchronize(ctx->st));
    return check_status(ctx);
}

// ---------------------------------------------------------------------------
// output_tot (code/output.F90:2494-3884): the .tot. variables sampled every
// istep nodes
// ---------------------------------------------------------------------------
// first and last node in [1, m] with (node + cum) divisible by istep (the
// reference's start/finish adjustment loops), and the count
static void out_axis(int m, long long cum, int istep, int &start, int &n) {
    auto md = [&](long long a) { return ((a % istep) + istep) % istep; };
    int s = 1, f = m;
    while (s <= m && md(s + cum) != 0) s++;
    while (f >= 1 && md(f + cum) != 0) f--;
    start = s;
    n = f >= s ? (f - s) / istep + 1 : 0;
}

static void out_grid(const tg_ctx *ctx, int istep, int start[3], int n[3]) {
    const Geom &g = ctx->g;
    out_axis(g.mx, ctx->P.mxcum, istep, start[0], n[0]);
    out_axis(g.my, ctx->P.mycum, istep, start[1], n[1]);
    if (g.dims == 3) out_axis(g.mz, ctx->P.mzcum, istep, start[2], n[2]);
    else {
        start[2] = 1;
        n[2] = 1;
    }
}

extern "C" int tg_output_dims(tg_ctx *ctx, int32_t istep, int32_t *dims) {
    if (!ctx || !dims || istep < 1) return TG_ERR_ARG;
    int start[3], n[3];
    out_grid(ctx, istep, start, n);
    for (int a = 0; a < 3; a++) dims[a] = n[a];
    return TG_OK;
}

extern "C" int tg_output_var(tg_ctx *ctx, int32_t var, int32_t istep, int32_t idx, int32_t idy, int32_t idz,
                             float *out) {
    if (!ctx || !out || istep < 1) return TG_ERR_ARG;
    const bool moment = var >= TG_OUT_MOMENT && var < TG_OUT_MOMENT + TG_MOMENT_KINDS;
    if (!(var >= TG_OUT_EX && var <= TG_OUT_JZ) && !moment)
        return fail(ctx, TG_ERR_ARG, "tg_output_var: variable %d unknown", var);
    if (moment && (idx < 0 || idy < 0 || idz < 0))
        return fail(ctx, TG_ERR_ARG, "tg_output_var: negative box half-width");
    int start[3], n[3];
    out_grid(ctx, istep, start, n);
    const size_t total = (size_t)n[0] * n[1] * n[2];
    if (total == 0) return TG_OK;
    const size_t lot = (size_t)ctx->g.lot;
    const float *src;
    int comp = -1;
    float add = 0.0f;
    if (moment) {
        if (!ctx->mom[0]) {
            int r = dalloc(ctx, &ctx->mom[0], lot);
            if (!r) r = dalloc(ctx, &ctx->mom[1], lot);
            if (r) return r;
            CK(cudaMemsetAsync(ctx->mom[0], 0, lot * 8, ctx->st));
            CK(cudaMemsetAsync(ctx->mom[1], 0, lot * 8, ctx->st));
        }
        long long cnt[2];
        int r = exact_counts(ctx, cnt);
        if (r) return r;
        float *f3[3] = {ctx->ftmp[0], ctx->ftmp[1], ctx->ftmp[2]};
        CK(launch_moments(ctx->g, ctx->P, ctx->sp[ctx->par], ctx->d_cnt + 2 * ctx->par, cnt[0] + cnt[1],
                          var - TG_OUT_MOMENT, idx, idy, ctx->g.dims == 3 ? idz : 0, ctx->mom[0], ctx->mom[1], f3,
                          ctx->st));
        src = f3[0];
    } else if (var <= TG_OUT_BZ) {
        comp = var - TG_OUT_EX;
        src = ctx->f[comp];
        // get_external_fields' constant values (zero when off)
        add = ctx->P.external_fields ? ctx->P.ext[comp] : 0.0f;
    } else {
        src = ctx->f[6 + (var - TG_OUT_JX)];
    }
    float *d_out = nullptr;
    CK(cudaMalloc(&d_out, total * 4));
    cudaError_t e = launch_output_sample(ctx->g, comp, src, add, start, n, istep, d_out, ctx->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d_out, total * 4, cudaMemcpyDeviceToHost, ctx->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
    cudaFree(d_out);
    if (e != cudaSuccess) return fail(ctx, TG_ERR_CUDA, "tg_output_var: %s", cudaGetErrorString(e));
    return check_status(ctx);
}

extern "C" int tg_output_particles(tg_ctx *ctx, int32_t species, int32_t stride, int64_t cap, float *vals,
                                   int32_t *ids, int64_t *count) {
    if (!ctx || !count || species < 0 || species > 1 || stride < 1 || cap < 0) return TG_ERR_ARG;
    if (cap > 0 && (!vals || !ids)) return TG_ERR_ARG;
    long long n[2];
    int r = exact_counts(ctx, n);
    if (r) return r;
    const long long m = n[species];
    *count = 0;
    if (m == 0) return TG_OK;
    if (m > INT32_MAX) return fail(ctx, TG_ERR_ARG, "tg_output_particles: species too large to scan");
    const Species &sp = ctx->sp[ctx->par][species];
    int *flag = nullptr, *pos = nullptr;
    void *tmp = nullptr;
    size_t tbytes = 0;
    float *d_vals = nullptr;
    int *d_ids = nullptr;
    cudaError_t e = cudaMalloc(&flag, (size_t)m * 4);
    if (e == cudaSuccess) e = cudaMalloc(&pos, (size_t)m * 4);
    if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(nullptr, tbytes, flag, pos, (int)m, ctx->st);
    if (e == cudaSuccess) e = cudaMalloc(&tmp, tbytes);
    if (e == cudaSuccess) e = launch_prt_flag(sp, m, stride, flag, ctx->st);
    if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(tmp, tbytes, flag, pos, (int)m, ctx->st);
    int last[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(&last[0], pos + m - 1, 4, cudaMemcpyDeviceToHost, ctx->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&last[1], flag + m - 1, 4, cudaMemcpyDeviceToHost, ctx->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
    const long long total = (long long)last[0] + last[1];
    if (e == cudaSuccess && total > 0 && total <= cap) {
        e = cudaMalloc(&d_vals, (size_t)total * 8 * 4);
        if (e == cudaSuccess) e = cudaMalloc(&d_ids, (size_t)total * 2 * 4);
        if (e == cudaSuccess) e = launch_prt_write(ctx->g, ctx->P, sp, m, flag, pos, total, d_vals, d_ids, ctx->st);
        // the device arrays are total long; the caller's are cap long
        for (int k = 0; k < 8 && e == cudaSuccess; k++)
            e = cudaMemcpyAsync(vals + (size_t)k * cap, d_vals + (size_t)k * total, (size_t)total * 4,
                                cudaMemcpyDeviceToHost, ctx->st);
        for (int k = 0; k < 2 && e == cudaSuccess; k++)
            e = cudaMemcpyAsync(ids + (size_t)k * cap, d_ids + (size_t)k * total, (size_t)total * 4,
                                cudaMemcpyDeviceToHost, ctx->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
    }
    cudaFree(flag);
    cudaFree(pos);
    cudaFree(tmp);
    cudaFree(d_vals);
    cudaFree(d_ids);
    if (e != cudaSuccess) return fail(ctx, TG_ERR_CUDA, "tg_output_particles: %s", cudaGetErrorString(e));
    *count = total;
    return check_status(ctx);
}

// ---------------------------------------------------------------------------
// flow-frame energy spectra (save_spectrum_2d, code/output.F90:794-1249)
// ---------------------------------------------------------------------------
extern "C" int tg_spectrum_dims(tg_ctx *ctx, int32_t gambins, int32_t *nxbins, int32_t *nybins) {
    if (!ctx || !nxbins || !nybins || gambins < 1) return TG_ERR_ARG;
    const SpecGrid sg = spec_grid(ctx->g.mx, ctx->g.my, ctx->g.ng, gambins);
    *nxbins = sg.nxb;
    *nybins = sg.nyb;
    return TG_OK;
}

// One spectrum pass over the slice grid sg: the gamma range over every
// particle, then per species the slice-mean velocities and the histograms
// (flow frame into rest[s], lab frame into lab[s] when given); with
// per_xgamma every bin is divided by its gamma - 1 (xgamma), as
// save_spectrum does. yslice may be NULL.
static int spectrum_run(tg_ctx *ctx, const SpecGrid &sg, float *const rest[2], float *const lab[2], float *xgamma,
                        float *xslice, float *yslice, float *gamma_range, bool per_xgamma, const char *who) {
    const int gambins = sg.gambins;
    const long long nsl = (long long)sg.nxb * sg.nyb;
    long long n[2];
    int r = exact_counts(ctx, n);
    if (r) return r;
    // scratch: 4 FP64 sums and 3 means per slice, the gamma range, the histograms
    double *acc = nullptr;
    float *mean = nullptr, *spec = nullptr;
    unsigned *range = nullptr;
    const size_t hbytes = (size_t)nsl * gambins * 4;
    cudaError_t e = cudaMalloc(&acc, (size_t)nsl * 4 * 8);
    if (e == cudaSuccess) e = cudaMalloc(&mean, (size_t)nsl * 3 * 4);
    if (e == cudaSuccess) e = cudaMalloc(&spec, 2 * hbytes);
    if (e == cudaSuccess) e = cudaMalloc(&range, 8);
    const unsigned one = 0x3f800000u;  // 1.0f
    const unsigned init[2] = {one, one};
    if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, (size_t)nsl * 4 * 8, ctx->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(range, init, 8, cudaMemcpyHostToDevice, ctx->st);
    if (e == cudaSuccess) e = launch_spec_range(ctx->sp[ctx->par], ctx->d_cnt + 2 * ctx->par, n[0] + n[1], range, ctx->st);
    unsigned got[2] = {one, one};
    if (e == cudaSuccess) e = cudaMemcpyAsync(got, range, 8, cudaMemcpyDeviceToHost, ctx->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
    float gmin, gmax;
    memcpy(&gmin, &got[0], 4);
    memcpy(&gmax, &got[1], 4);
    const float gammin = fmaxf(gmin, 1.0f + 1e-6f);
    const float lg0 = log10_single(gammin - 1.0f);
    const float dgam = (log10_single(gmax - 1.0f) - lg0) / (float)gambins;
    for (int i = 1; i <= gambins; i++) xgamma[i - 1] = powf(10.0f, (float)(i - 1) * dgam + lg0);
    for (int i = 1; i <= sg.nxb; i++) xslice[i - 1] = sg.dxslice * (float)(i - 1) + 0.5f * sg.dxslice + (float)sg.mxmin;
    if (yslice)
        for (int i = 1; i <= sg.nyb; i++)
            yslice[i - 1] = sg.dyslice * (float)(i - 1) + 0.5f * sg.dyslice + (float)sg.mymin;
    if (gamma_range) {
        gamma_range[0] = gammin;
        gamma_range[1] = gmax;
    }
    for (int s = 0; s < 2 && e == cudaSuccess; s++) {
        float *spec_lab = lab[s] ? spec + (size_t)nsl * gambins : nullptr;
        e = cudaMemsetAsync(spec, 0, 2 * hbytes, ctx->st);
        if (e == cudaSuccess)
            e = launch_spec_species(ctx->g, ctx->P, sg, ctx->sp[ctx->par][s], ctx->d_cnt + 2 * ctx->par + s,
                                    n[s], acc, mean, lg0, dgam, spec, spec_lab, ctx->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(rest[s], spec, hbytes, cudaMemcpyDeviceToHost, ctx->st);
        if (e == cudaSuccess && lab[s]) e = cudaMemcpyAsync(lab[s], spec_lab, hbytes, cudaMemcpyDeviceToHost, ctx->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->st);
        if (e == cudaSuccess && per_xgamma)
            for (long long t = 0; t < nsl * gambins; t++) {
                rest[s][t] = rest[s][t] / xgamma[t / nsl];
                if (lab[s]) lab[s][t] = lab[s][t] / xgamma[t / nsl];
            }
    }
    cudaFree(acc);
    cudaFree(mean);
    cudaFree(spec);
    cudaFree(range);
    if (e != cudaSuccess) return fail(ctx, TG_ERR_CUDA, "%s: %s", who, cudaGetErrorString(e));
    return check_status(ctx);
}

extern "C" int tg_spectrum(tg_ctx *ctx, int32_t gambins, float *spec_ions, float *spec_lecs, float *xgamma,
                           float *xslice, float *yslice, float *gamma_range) {
    if (!ctx || !spec_ions || !spec_lecs || !xgamma || !xslice || !yslice || gambins < 1) return TG_ERR_ARG;
    const SpecGrid sg = spec_grid(ctx->g.mx, ctx->g.my, ctx->g.ng, gambins);
    float *rest[2] = {spec_ions, spec_lecs}, *lab[2] = {nullptr, nullptr};
    return spectrum_run(ctx, sg, rest, lab, xgamma, xslice, yslice, gamma_range, false, "tg_spectrum");
}

extern "C" int tg_spectrum_x_bins(tg_ctx *ctx, int32_t *nbins) {
    if (!ctx || !nbins) return TG_ERR_ARG;
    *nbins = spec_grid_x(ctx->g.mx, 1).nxb;
    return TG_OK;
}

extern "C" int tg_spectrum_x(tg_ctx *ctx, int32_t gambins, float *spec_ions, float *spec_lecs, float *spec_ions_rest,
                             float *spec_lecs_rest, float *xgamma, float *xslice, float *gamma_range) {
    if (!ctx || !spec_ions || !spec_lecs || !spec_ions_rest || !spec_lecs_rest || !xgamma || !xslice || gambins < 1)
        return TG_ERR_ARG;
    const SpecGrid sg = spec_grid_x(ctx->g.mx, gambins);
    float *rest[2] = {spec_ions_rest, spec_lecs_rest}, *lab[2] = {spec_ions, spec_lecs};
    return spectrum_run(ctx, sg, rest, lab, xgamma, xslice, nullptr, gamma_range, true, "tg_spectrum_x");
}

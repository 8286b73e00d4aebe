// Batched ensemble of the GB300 TRISTAN-MP hot path (sm_103a): many
// independent periodic 2D boxes of uneven size (seed or parameter
// ensembles) stepped together, one launch per phase for all boxes, the laps
// replayed from a captured CUDA graph.
//
// Layout: every field array of every box lives in one concatenated buffer
// per component (box b at element offset fofs[b], 64-element aligned); the
// particles of all boxes share one SoA buffer per species, kept sorted by a
// global tile key (box-major: box b owns tiles tofs[b] .. tofs[b+1]-1), so
// one counting sort over all tiles keeps every box's particles together and
// grouped by tile. Field kernels run the same per-cell functions as the
// single-domain kernels over a block table (each CTA takes one chunk of one
// box); the particle kernels are persistent, one per shape order on
// concurrent graph branches: one CTA per resident slot pulls tiles from its
// order's work queue (largest boxes first). Per cell and per particle the
// arithmetic is that of the single-domain path, so in fixed-point mode every
// box gives the bits a single-domain run of the same box gives.
//
// No counterpart in the reference, which runs one domain per job: each box
// is what one run of the reference's main loop (code/tristanmainloop.F90:
// 117-303) steps.
#include <cuda_runtime.h>

#include <mutex>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "tg_fields.cuh"
#include "tg_particles.cuh"

using namespace tg;

namespace tg {

#define TG_ENS_CHUNK 4096   // cells per CTA of a batched field kernel
#define TG_ENS_DIAG_CAP 8   // diagnostics records kept per box
// resident CTAs per SM of the persistent tile kernels (as the 2D tile kernel)
#ifndef TG_ENS_MINB
#define TG_ENS_MINB TG_TILES_MINB_2D
#endif

// per-box constants of the batched field kernels
struct EnsBox {
    Geom g;
    long long fofs;   // element offset of the box in the concatenated arrays
    GhostAxis gax[3];
    long long gn[3];  // ghost cells per part of a bc_b1 / bc_e1 pass
    Box bb, be;       // advance_b / advance_e update ranges
    float cstb, cste;
    int q5;
    double fx_inv;
};

enum { EK_GHOST = 0, EK_ADVB, EK_ADVE, EK_FOLD0, EK_FOLD1, EK_LOT, EK_N };

__device__ __forceinline__ long long ens_chunk_end(long long t0, long long n) {
    return t0 + TG_ENS_CHUNK < n ? t0 + TG_ENS_CHUNK : n;
}

__global__ void __launch_bounds__(256) k_ens_ghost(const EnsBox *__restrict__ boxes, const int2 *__restrict__ blk,
                                                   float *a, float *b, float *c) {
    const int2 w = blk[blockIdx.x];
    const EnsBox &B = boxes[w.x];
    const long long t0 = (long long)w.y * TG_ENS_CHUNK;
    const long long t1 = ens_chunk_end(t0, B.gn[0] + B.gn[1] + B.gn[2]);
    const long long o = B.fofs;
    for (long long t = t0 + threadIdx.x; t < t1; t += blockDim.x)
        ghost_one(B.g, a + o, b + o, c + o, B.gax[0], B.gax[1], B.gax[2], B.gn[0], B.gn[1], t);
}

__global__ void __launch_bounds__(256) k_ens_advance_b(const EnsBox *__restrict__ boxes, const int2 *__restrict__ blk,
                                                       float *const *__restrict__ f9) {
    const int2 w = blk[blockIdx.x];
    const EnsBox &B = boxes[w.x];
    const long long t0 = (long long)w.y * TG_ENS_CHUNK;
    const long long t1 = ens_chunk_end(t0, (long long)B.bb.ni * B.bb.nj * B.bb.nk);
    const long long o = B.fofs;
    for (long long t = t0 + threadIdx.x; t < t1; t += blockDim.x)
        advance_b_one<2>(B.g, B.bb, B.cstb, f9[0] + o, f9[1] + o, f9[2] + o, f9[3] + o, f9[4] + o, f9[5] + o, t);
}

__global__ void __launch_bounds__(256) k_ens_advance_e(const EnsBox *__restrict__ boxes, const int2 *__restrict__ blk,
                                                       float *const *__restrict__ f9) {
    const int2 w = blk[blockIdx.x];
    const EnsBox &B = boxes[w.x];
    const long long t0 = (long long)w.y * TG_ENS_CHUNK;
    const long long t1 = ens_chunk_end(t0, (long long)B.be.ni * B.be.nj * B.be.nk);
    const long long o = B.fofs;
    for (long long t = t0 + threadIdx.x; t < t1; t += blockDim.x)
        advance_e_one<2>(B.g, B.be, B.cste, f9[0] + o, f9[1] + o, f9[2] + o, f9[3] + o, f9[4] + o, f9[5] + o, t);
}

__global__ void __launch_bounds__(256) k_ens_fold(const EnsBox *__restrict__ boxes, const int2 *__restrict__ blk,
                                                  int axis, float *cx, float *cy, float *cz) {
    const int2 w = blk[blockIdx.x];
    const EnsBox &B = boxes[w.x];
    const long long t0 = (long long)w.y * TG_ENS_CHUNK;
    const long long t1 = ens_chunk_end(t0, fold_cells(B.g, axis));
    const long long o = B.fofs;
    const int m = axis == 0 ? B.g.mx : B.g.my;
    const int q5 = axis == 1 ? B.q5 : 0;
    for (long long t = t0 + threadIdx.x; t < t1; t += blockDim.x)
        fold_one(B.g, axis, m, B.g.ng, cx + o, cy + o, cz + o, q5, t);
}

__global__ void __launch_bounds__(256) k_ens_filter(const EnsBox *__restrict__ boxes, const int2 *__restrict__ blk,
                                                    const float *i0, const float *i1, const float *i2, float *o0,
                                                    float *o1, float *o2) {
    const int2 w = blk[blockIdx.x];
    const EnsBox &B = boxes[w.x];
    const long long t0 = (long long)w.y * TG_ENS_CHUNK;
    const long long t1 = ens_chunk_end(t0, B.g.lot);
    const long long o = B.fofs;
    for (long long t = t0 + threadIdx.x; t < t1; t += blockDim.x)
        filter_one<2>(B.g, i0 + o, i1 + o, i2 + o, o0 + o, o1 + o, o2 + o, t);
}

__global__ void __launch_bounds__(256) k_ens_fixed_to_float(const EnsBox *__restrict__ boxes,
                                                            const int2 *__restrict__ blk,
                                                            unsigned long long *const *__restrict__ fx,
                                                            float *const *__restrict__ f9) {
    const int2 w = blk[blockIdx.x];
    const EnsBox &B = boxes[w.x];
    const long long t0 = (long long)w.y * TG_ENS_CHUNK;
    const long long t1 = ens_chunk_end(t0, B.g.lot);
    const long long o = B.fofs;
    for (long long t = t0 + threadIdx.x; t < t1; t += blockDim.x)
        fixed_to_float_one(B.fx_inv, fx[0] + o, fx[1] + o, fx[2] + o, f9[6] + o, f9[7] + o, f9[8] + o, t);
}

// Persistent particle kernel of one shape order: tiles pulled from that
// order's work queue; a CTA keeps the arguments of its current box in
// shared memory. The three orders run as concurrent branches of the lap.
template <int ORDER, bool FIXED>
__global__ void __launch_bounds__(256, TG_ENS_MINB)
    k_ens_tiles(const TileArgs *__restrict__ boxes, const int2 *__restrict__ work, int nwork, int *queue) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ __align__(16) TileArgs sa;
    __shared__ int s_item;
    int cur = -1;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
        __syncthreads();
        const int wi = s_item;
        if (wi >= nwork) break;  // uniform across the CTA
        const int2 it = work[wi];
        if (it.x != cur) {
            const int *src = reinterpret_cast<const int *>(boxes + it.x);
            int *dst = reinterpret_cast<int *>(&sa);
            for (int t = threadIdx.x; t < (int)(sizeof(TileArgs) / 4); t += blockDim.x) dst[t] = src[t];
            cur = it.x;
        }
        __syncthreads();
        tile_body<2, ORDER, FIXED, true, true>(sa, it.y, smem_raw);
        __syncthreads();  // window and arguments free for the next tile
    }
}

// The same kernel reading its box's arguments from a constant-memory table
// (the arguments are uniform across the CTA, so every read is a broadcast
// from the constant cache). With the arguments in shared memory the deposit
// loop re-reads them there and the kernel ran 1.2x slower per particle than
// the single-domain one. The table holds up to TG_ENS_CONST_BOXES boxes; it
// is one per device, shared by every ensemble of the process (see
// claim_const_table); larger ensembles use k_ens_tiles.
#define TG_ENS_CONST_BOXES 72
__constant__ TileArgs c_ens_targs[TG_ENS_CONST_BOXES];
template <int ORDER, bool FIXED>
__global__ void __launch_bounds__(256, TG_ENS_MINB)
    k_ens_tiles_c(const int2 *__restrict__ work, int nwork, int *queue) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(queue, 1);
        __syncthreads();
        const int wi = s_item;
        if (wi >= nwork) break;  // uniform across the CTA
        const int2 it = work[wi];
        tile_body<2, ORDER, FIXED, true, true>(c_ens_targs[it.x], it.y, smem_raw);
        __syncthreads();  // window free for the next tile
    }
}

// tile counting sort over all boxes: one flat grid over the particles of
// every box (stored box after box), so a large box gets as many threads as
// its particles need; a particle's box is found by bisection of the box
// starts (the last box whose start is at or before it: empty boxes skipped)
__device__ __forceinline__ int ens_box_of(const long long *__restrict__ bstart, int nbox, long long n) {
    int lo = 0, hi = nbox;  // bstart[lo] <= n < bstart[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(bstart + mid) <= n) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void k_ens_count(const Geom *__restrict__ geoms, Species sp, const long long *__restrict__ bstart, int nbox,
                            const int *__restrict__ tofs, int *hist) {
    const long long total = bstart[nbox];
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < total;
         n += (long long)gridDim.x * blockDim.x) {
        const int cell = sp.cell[n];
        if (cell < 0) continue;
        const int b = ens_box_of(bstart, nbox, n);
        const Geom &g = geoms[b];
        int i, j, k;
        cell_ijk(g, cell, i, j, k);
        agg_inc(hist, tofs[b] + tile_of(g, i, j, k));
    }
}

__global__ void k_ens_scatter(const Geom *__restrict__ geoms, Species src, Species dst,
                              const long long *__restrict__ bstart, int nbox, const int *__restrict__ tofs,
                              const int *start, int *cursor) {
    // read order and early loads as in k_tile_scatter
    constexpr int S = TG_SCATTER_STRIDE, B = 32 * S;
    const long long total = bstart[nbox];
    const long long mmax = (total + B - 1) / B * B;
    for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < mmax;
         m += (long long)gridDim.x * blockDim.x) {
        const int q = (int)(m % B);
        const long long n = m - q + (q & 31) * S + (q >> 5);
        if (n >= total) continue;
        const int cell = src.cell[n];
        if (cell < 0) continue;
        const float ox = src.ox[n], oy = src.oy[n], oz = src.oz[n];
        const float u = src.u[n], v = src.v[n], w = src.w[n], ch = src.ch[n];
        const int32_t ind = src.ind[n], proc = src.proc[n], spl = src.splitlev[n];
        const int b = ens_box_of(bstart, nbox, n);
        const Geom &g = geoms[b];
        int i, j, k;
        cell_ijk(g, cell, i, j, k);
        const int t = tofs[b] + tile_of(g, i, j, k);
        const long long d = (long long)start[t] + agg_inc(cursor, t);
        dst.cell[d] = cell;
        dst.ox[d] = ox;
        dst.oy[d] = oy;
        dst.oz[d] = oz;
        dst.u[d] = u;
        dst.v[d] = v;
        dst.w[d] = w;
        dst.ch[d] = ch;
        dst.ind[d] = ind;
        dst.proc[d] = proc;
        dst.splitlev[d] = spl;
    }
}

// first particle of every box after a scan: start of its first tile
__global__ void k_ens_bstart(const int *__restrict__ tofs, const int *__restrict__ start, long long *bnext,
                             int nbox) {
    for (int b = threadIdx.x; b <= nbox; b += blockDim.x) bnext[b] = start[tofs[b]];
}

}  // namespace tg

// ---------------------------------------------------------------------------
// ensemble context
// ---------------------------------------------------------------------------
struct tg_ens {
    int nbox = 0;
    std::vector<tg_config> cfg;
    std::vector<Geom> g;
    std::vector<Params> P;
    std::vector<long long> fofs;  // [nbox + 1]
    std::vector<int> tofs;        // [nbox + 1]
    long long ncell = 0;          // concatenated field elements
    int T = 0;                    // tiles of all boxes
    long long capacity = 0;       // particles per species, all boxes
    bool fixed = false;
    int sort_every = 1, ntimes = 4;
    size_t smem = 0;
    int tile_grid[3] = {0, 0, 0};  // per shape order
    bool use_const = false;        // tile arguments from the constant-memory table
    cudaEvent_t laps_done = nullptr;  // after the last tg_ens_step's laps
    cudaStream_t st = nullptr;
    int device = 0;
    float *f[9] = {};
    float *ftmp[3] = {};
    unsigned long long *fix[3] = {};
    float **d_f9 = nullptr;
    unsigned long long **d_fx3 = nullptr;
    Species sp[2][2];
    int par = 0;
    long long *d_cnt = nullptr;           // [parity][species] totals
    long long *bstart[2][2] = {};         // [parity][species][nbox + 1]
    std::vector<long long> hbstart[2];    // host copy per species of the current parity
    int *tstart[2] = {}, *hist[2] = {}, *cursor[2] = {};
    int *d_status = nullptr;
    int *queue = nullptr;
    EnsBox *d_box = nullptr;
    Geom *d_geom = nullptr;
    int *d_tofs = nullptr;
    TileArgs *d_targs = nullptr;  // [parity][count tiles][box]
    int2 *d_work = nullptr;
    int wstart[3] = {0, 0, 0}, nwork[3] = {0, 0, 0};  // per shape order: segment of d_work
    cudaStream_t side[2] = {nullptr, nullptr};       // branches for orders 2 and 1
    cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
    int2 *d_blk[EK_N] = {};
    int nblk[EK_N] = {};
    // host bindings
    std::vector<float *> hf;  // [box][9]
    std::vector<void *> hp;
    std::vector<int32_t *> hions, hlecs;
    unsigned char *stage = nullptr;
    // FP64 diagnostics (scratch sized for the largest box)
    unsigned long long *rhofx = nullptr;
    double *rho[2] = {};
    double *dacc = nullptr, *dhist = nullptr;
    unsigned long long *dcounter = nullptr;
    // graphs: one cycle of 2*sort_every laps per starting parity
    cudaGraphExec_t cycle[2] = {nullptr, nullptr};
    int kernels_per_step = 0;
    bool dirty = true;
    bool may_have_dead = false;
    long long lap = 0;
    char err[512] = {0};
    std::vector<void *> allocs;
};

static thread_local char g_ens_error[512];

// The constant-memory table of tile arguments is one per device and shared
// by every ensemble of the process: each lap copies its boxes' arguments
// into it before its tile kernels. An ensemble that steps after another
// one on the same device first makes its stream wait for the other's last
// laps (an event), so their laps never overlap on the table.
#define TG_ENS_MAX_DEVICES 64
static std::mutex g_const_mu;
static tg_ens *g_const_owner[TG_ENS_MAX_DEVICES] = {};

static int efail(tg_ens *E, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    snprintf(E ? E->err : g_ens_error, 512, "%s", buf);
    return code;
}

#define ECK(call)                                                                                     \
    do {                                                                                              \
        cudaError_t e__ = (call);                                                                     \
        if (e__ != cudaSuccess)                                                                       \
            return efail(E, TG_ERR_CUDA, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e__),     \
                         __FILE__, __LINE__);                                                         \
    } while (0)

template <class T>
static int ealloc(tg_ens *E, T **p, size_t n) {
    void *q = nullptr;
    ECK(cudaMalloc(&q, n * sizeof(T) + 256));
    E->allocs.push_back(q);
    *p = (T *)q;
    return TG_OK;
}

static Species sp_at(const Species &s, long long o) {
    Species r = s;
    r.cell += o;
    r.ox += o;
    r.oy += o;
    r.oz += o;
    r.u += o;
    r.v += o;
    r.w += o;
    r.ch += o;
    r.ind += o;
    r.proc += o;
    r.splitlev += o;
    return r;
}

static int alloc_species(tg_ens *E, Species &s, size_t n) {
    int r;
    if ((r = ealloc(E, &s.cell, n))) return r;
    if ((r = ealloc(E, &s.ox, n))) return r;
    if ((r = ealloc(E, &s.oy, n))) return r;
    if ((r = ealloc(E, &s.oz, n))) return r;
    if ((r = ealloc(E, &s.u, n))) return r;
    if ((r = ealloc(E, &s.v, n))) return r;
    if ((r = ealloc(E, &s.w, n))) return r;
    if ((r = ealloc(E, &s.ch, n))) return r;
    if ((r = ealloc(E, &s.ind, n))) return r;
    if ((r = ealloc(E, &s.proc, n))) return r;
    if ((r = ealloc(E, &s.splitlev, n))) return r;
    return TG_OK;
}

static int check_status(tg_ens *E) {
    int st = 0;
    ECK(cudaMemcpyAsync(&st, E->d_status, sizeof(int), cudaMemcpyDeviceToHost, E->st));
    ECK(cudaStreamSynchronize(E->st));
    if (st == 0) return TG_OK;
    ECK(cudaMemsetAsync(E->d_status, 0, sizeof(int), E->st));
    if (st & ST_NAN) return efail(E, TG_ERR_NAN, "non-finite particle coordinate (device status %d)", st);
    if (st & ST_OVERFLOW) return efail(E, TG_ERR_OVERFLOW, "particle capacity exceeded (device status %d)", st);
    if (st & ST_CHARGE_GRID)
        return efail(E, TG_ERR_OVERFLOW, "diagnostics: a node holds 2^17 particle charges or more (device status %d)", st);
    return efail(E, TG_ERR_BOUNDS, "particle or deposit outside its box (device status %d)", st);
}

// block table of one batched field kernel: CTA -> (box, chunk)
static int make_blocks(tg_ens *E, int kind, const std::vector<long long> &cells) {
    std::vector<int2> blk;
    for (int b = 0; b < E->nbox; b++) {
        const long long nch = (cells[b] + TG_ENS_CHUNK - 1) / TG_ENS_CHUNK;
        for (long long c = 0; c < nch; c++) blk.push_back(make_int2(b, (int)c));
    }
    if (blk.empty()) blk.push_back(make_int2(0, 1 << 30));  // one CTA with an empty range
    E->nblk[kind] = (int)blk.size();
    int r = ealloc(E, &E->d_blk[kind], blk.size());
    if (r) return r;
    ECK(cudaMemcpy(E->d_blk[kind], blk.data(), blk.size() * sizeof(int2), cudaMemcpyHostToDevice));
    return TG_OK;
}

static TileArgs ens_tile_args(tg_ens *E, int b, int par, bool count_tiles) {
    TileArgs a;
    memset(&a, 0, sizeof a);
    const long long o = E->fofs[b];
    a.g = E->g[b];
    a.P = E->P[b];
    a.f.ex = E->f[0] + o; a.f.ey = E->f[1] + o; a.f.ez = E->f[2] + o;
    a.f.bx = E->f[3] + o; a.f.by = E->f[4] + o; a.f.bz = E->f[5] + o;
    for (int s = 0; s < 2; s++) {
        a.sp[s] = E->sp[par][s];
        a.tstart[s] = E->tstart[s] + E->tofs[b];
        a.newcount[s] = count_tiles ? E->hist[s] + E->tofs[b] : nullptr;
    }
    for (int cc = 0; cc < 3; cc++) {
        a.cur[cc] = E->f[6 + cc] + o;
        a.fix[cc] = E->fixed ? E->fix[cc] + o : nullptr;
    }
    a.status = E->d_status;
    return a;
}

extern "C" void tg_ens_finalize(tg_ens *E);

extern "C" int tg_ens_init(const tg_config *cfgs, int32_t nbox, tg_ens **out) {
    tg_ens *E = nullptr;
    if (!cfgs || !out || nbox < 1) return efail(nullptr, TG_ERR_ARG, "tg_ens_init: null argument or nbox < 1");
    *out = nullptr;
    E = new (std::nothrow) tg_ens();
    if (!E) return efail(nullptr, TG_ERR_ARG, "tg_ens_init: out of host memory");
    E->nbox = nbox;
    E->cfg.assign(cfgs, cfgs + nbox);
    E->g.resize(nbox);
    E->P.resize(nbox);
    int r = TG_OK;
    for (int b = 0; b < nbox && !r; b++) {
        const tg_config &c = cfgs[b];
        char why[256] = {0};
        if (c.dims != 2) r = efail(E, TG_ERR_ARG, "box %d: ensemble boxes are 2D", b);
        else if (!c.periodic[0] || !c.periodic[1]) r = efail(E, TG_ERR_ARG, "box %d: ensemble boxes are periodic", b);
        else if (c.deposit_mode != cfgs[0].deposit_mode)
            r = efail(E, TG_ERR_ARG, "box %d: all boxes use the same deposit mode", b);
        else if ((c.sort_every < 1 ? 1 : c.sort_every) != (cfgs[0].sort_every < 1 ? 1 : cfgs[0].sort_every))
            r = efail(E, TG_ERR_ARG, "box %d: all boxes use the same sort cadence", b);
        else if (c.ntimes != cfgs[0].ntimes) r = efail(E, TG_ERR_ARG, "box %d: all boxes use the same ntimes", b);
        else if (c.device != cfgs[0].device) r = efail(E, TG_ERR_ARG, "box %d: all boxes on one device", b);
        else if (c.maxhlf <= 0 || c.maxhlf >= (1LL << 31))
            r = efail(E, TG_ERR_ARG, "box %d: maxhlf must be in [1, 2^31)", b);
        else if (build_geom(c, E->g[b], why, sizeof why) != TG_OK)
            r = efail(E, TG_ERR_ARG, "box %d: %s", b, why);
        // the batched fold adds both ghost slabs of an axis in one launch,
        // which needs disjoint target slabs: nghost interior cells per axis
        else if (!fold_in_one_pass(E->g[b], 0) || !fold_in_one_pass(E->g[b], 1))
            r = efail(E, TG_ERR_ARG, "box %d: ensemble boxes need at least %d interior cells per axis", b,
                      E->g[b].ng);
        if (!r) build_params(c, E->P[b]);
    }
    if (r) {
        snprintf(g_ens_error, sizeof g_ens_error, "%s", E->err);
        delete E;
        return r;
    }
    E->fixed = cfgs[0].deposit_mode == TG_DEPOSIT_FIXED;
    E->sort_every = cfgs[0].sort_every < 1 ? 1 : cfgs[0].sort_every;
    E->ntimes = cfgs[0].ntimes;
    E->device = cfgs[0].device;
    // offsets
    E->fofs.resize(nbox + 1);
    E->tofs.resize(nbox + 1);
    long long fo = 0, cap = 0, maxcap = 0, maxint = 0;
    int to = 0, maxw = 0;
    for (int b = 0; b < nbox; b++) {
        E->fofs[b] = fo;
        fo += (E->g[b].lot + 63) / 64 * 64;
        E->tofs[b] = to;
        to += E->g[b].ntiles;
        cap += cfgs[b].maxhlf;
        maxcap = std::max(maxcap, (long long)cfgs[b].maxhlf);
        maxw = std::max(maxw, E->g[b].wcells);
        maxint = std::max(maxint, (long long)(E->g[b].mx - E->g[b].ng) * (E->g[b].my - E->g[b].ng));
    }
    E->fofs[nbox] = fo;
    E->tofs[nbox] = to;
    E->ncell = fo;
    E->T = to;
    E->capacity = cap;
    E->smem = tile_smem_bytes(2, maxw, 0);
    if (cap >= (1LL << 31)) {
        delete E;
        return efail(nullptr, TG_ERR_ARG, "tg_ens_init: %lld particles per species exceed int32 indices", cap);
    }
    cudaError_t e = cudaSetDevice(E->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&E->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        efail(nullptr, TG_ERR_CUDA, "tg_ens_init: CUDA device %d unavailable: %s", E->device, cudaGetErrorString(e));
        delete E;
        return TG_ERR_CUDA;
    }
    const size_t n = (size_t)E->ncell;
    for (int a = 0; a < 9 && !r; a++) r = ealloc(E, &E->f[a], n);
    for (int a = 0; a < 3 && !r; a++) r = ealloc(E, &E->ftmp[a], n);
    if (E->fixed)
        for (int a = 0; a < 3 && !r; a++) r = ealloc(E, &E->fix[a], n);
    for (int p = 0; p < 2 && !r; p++)
        for (int s = 0; s < 2 && !r; s++) {
            r = alloc_species(E, E->sp[p][s], (size_t)cap);
            if (!r) r = ealloc(E, &E->bstart[p][s], (size_t)nbox + 1);
        }
    if (!r) r = ealloc(E, &E->d_cnt, 4);
    for (int s = 0; s < 2 && !r; s++) {
        r = ealloc(E, &E->tstart[s], (size_t)E->T + 1);
        if (!r) r = ealloc(E, &E->hist[s], (size_t)E->T);
        if (!r) r = ealloc(E, &E->cursor[s], (size_t)E->T);
    }
    if (!r) r = ealloc(E, &E->d_status, 1);
    if (!r) r = ealloc(E, &E->queue, 3);
    if (!r) r = ealloc(E, &E->d_box, (size_t)nbox);
    if (!r) r = ealloc(E, &E->d_geom, (size_t)nbox);
    if (!r) r = ealloc(E, &E->d_tofs, (size_t)nbox + 1);
    if (!r) r = ealloc(E, &E->d_targs, (size_t)4 * nbox);
    if (!r) r = ealloc(E, &E->d_work, (size_t)E->T);
    if (!r) r = ealloc(E, &E->d_f9, 9);
    if (!r) r = ealloc(E, &E->d_fx3, 3);
    if (!r) r = ealloc(E, &E->rhofx, (size_t)maxint);
    if (!r) r = ealloc(E, &E->rho[0], (size_t)maxint);
    if (!r) r = ealloc(E, &E->rho[1], (size_t)maxint);
    if (!r) r = ealloc(E, &E->dacc, (size_t)nbox * 16);
    if (!r) r = ealloc(E, &E->dhist, (size_t)nbox * TG_ENS_DIAG_CAP * 16);
    if (!r) r = ealloc(E, &E->dcounter, (size_t)nbox);
    if (!r) r = ealloc(E, &E->stage, (size_t)maxcap * 40);
    // per-box tables
    if (!r) {
        std::vector<EnsBox> boxes(nbox);
        std::vector<long long> cells[EK_N];
        for (int k = 0; k < EK_N; k++) cells[k].resize(nbox);
        for (int b = 0; b < nbox; b++) {
            EnsBox &B = boxes[b];
            memset(&B, 0, sizeof B);
            const Geom &g = E->g[b];
            B.g = g;
            B.fofs = E->fofs[b];
            ghost_plan(g, GHOST_BC, B.gax, B.gn);
            int i2, j2, k2;
            b_range(g, 0, B.bb.i1, i2);
            b_range(g, 1, B.bb.j1, j2);
            b_range(g, 2, B.bb.k1, k2);
            B.bb.ni = i2 - B.bb.i1 + 1;
            B.bb.nj = j2 - B.bb.j1 + 1;
            B.bb.nk = k2 - B.bb.k1 + 1;
            e_range(g, 0, B.be.i1, i2);
            e_range(g, 1, B.be.j1, j2);
            e_range(g, 2, B.be.k1, k2);
            B.be.ni = i2 - B.be.i1 + 1;
            B.be.nj = j2 - B.be.j1 + 1;
            B.be.nk = k2 - B.be.k1 + 1;
            B.cstb = E->P[b].corr * (0.5f * E->P[b].c);
            B.cste = E->P[b].corr * E->P[b].c;
            B.q5 = (E->P[b].quirks & TG_QUIRK_Q5_LHS) ? 1 : 0;
            B.fx_inv = E->P[b].fx_inv;
            cells[EK_GHOST][b] = B.gn[0] + B.gn[1] + B.gn[2];
            cells[EK_ADVB][b] = (long long)B.bb.ni * B.bb.nj * B.bb.nk;
            cells[EK_ADVE][b] = (long long)B.be.ni * B.be.nj * B.be.nk;
            cells[EK_FOLD0][b] = fold_cells(g, 0);
            cells[EK_FOLD1][b] = fold_cells(g, 1);
            cells[EK_LOT][b] = g.lot;
        }
        for (int k = 0; k < EK_N && !r; k++) r = make_blocks(E, k, cells[k]);
        if (!r) {
            e = cudaMemcpy(E->d_box, boxes.data(), nbox * sizeof(EnsBox), cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = cudaMemcpy(E->d_geom, E->g.data(), nbox * sizeof(Geom), cudaMemcpyHostToDevice);
            if (e == cudaSuccess)
                e = cudaMemcpy(E->d_tofs, E->tofs.data(), (nbox + 1) * sizeof(int), cudaMemcpyHostToDevice);
            std::vector<TileArgs> ta((size_t)4 * nbox);
            for (int p = 0; p < 2; p++)
                for (int cnt = 0; cnt < 2; cnt++)
                    for (int b = 0; b < nbox; b++) ta[(size_t)(p * 2 + cnt) * nbox + b] = ens_tile_args(E, b, p, cnt);
            if (e == cudaSuccess)
                e = cudaMemcpy(E->d_targs, ta.data(), ta.size() * sizeof(TileArgs), cudaMemcpyHostToDevice);
            float *f9[9];
            for (int a = 0; a < 9; a++) f9[a] = E->f[a];
            if (e == cudaSuccess) e = cudaMemcpy(E->d_f9, f9, sizeof f9, cudaMemcpyHostToDevice);
            unsigned long long *fx3[3] = {E->fix[0], E->fix[1], E->fix[2]};
            if (e == cudaSuccess) e = cudaMemcpy(E->d_fx3, fx3, sizeof fx3, cudaMemcpyHostToDevice);
            if (e != cudaSuccess) r = efail(E, TG_ERR_CUDA, "tg_ens_init: %s", cudaGetErrorString(e));
        }
    }
    // persistent grid of the particle kernel: every resident slot
    if (!r) {
        int nsm = 0, per_sm = 1;
        void (*kerns[3])(const TileArgs *, const int2 *, int, int *);
        if (E->fixed) {
            kerns[0] = k_ens_tiles<1, true>;
            kerns[1] = k_ens_tiles<2, true>;
            kerns[2] = k_ens_tiles<3, true>;
        } else {
            kerns[0] = k_ens_tiles<1, false>;
            kerns[1] = k_ens_tiles<2, false>;
            kerns[2] = k_ens_tiles<3, false>;
        }
        e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, E->device);
        for (int o = 0; o < 3 && e == cudaSuccess && per_sm >= 1; o++) {
            e = cudaFuncSetAttribute(kerns[o], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)E->smem);
            if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kerns[o], 256, E->smem);
            E->tile_grid[o] = nsm * per_sm;
        }
        void (*kc[3])(const int2 *, int, int *);
        if (E->fixed) {
            kc[0] = k_ens_tiles_c<1, true>;
            kc[1] = k_ens_tiles_c<2, true>;
            kc[2] = k_ens_tiles_c<3, true>;
        } else {
            kc[0] = k_ens_tiles_c<1, false>;
            kc[1] = k_ens_tiles_c<2, false>;
            kc[2] = k_ens_tiles_c<3, false>;
        }
        for (int o = 0; o < 3 && e == cudaSuccess; o++)
            e = cudaFuncSetAttribute(kc[o], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)E->smem);
        E->use_const = E->nbox <= TG_ENS_CONST_BOXES && E->device >= 0 && E->device < TG_ENS_MAX_DEVICES;
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E->laps_done, cudaEventDisableTiming);
        for (int b = 0; b < 2 && e == cudaSuccess; b++) {
            e = cudaStreamCreateWithFlags(&E->side[b], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E->join[b], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&E->fork, cudaEventDisableTiming);
        if (e != cudaSuccess) r = efail(E, TG_ERR_CUDA, "tg_ens_init: %s", cudaGetErrorString(e));
        else if (per_sm < 1) r = efail(E, TG_ERR_ARG, "tg_ens_init: deposit window of %zu bytes does not fit", E->smem);
    }
    if (!r) {
        cudaStream_t st = E->st;
        for (int a = 0; a < 9; a++) e = e != cudaSuccess ? e : cudaMemsetAsync(E->f[a], 0, n * 4, st);
        for (int a = 0; a < 3; a++) e = e != cudaSuccess ? e : cudaMemsetAsync(E->ftmp[a], 0, n * 4, st);
        if (E->fixed)
            for (int a = 0; a < 3; a++) e = e != cudaSuccess ? e : cudaMemsetAsync(E->fix[a], 0, n * 8, st);
        for (int s = 0; s < 2; s++) {
            if (e == cudaSuccess) e = cudaMemsetAsync(E->tstart[s], 0, ((size_t)E->T + 1) * 4, st);
            if (e == cudaSuccess) e = cudaMemsetAsync(E->hist[s], 0, (size_t)E->T * 4, st);
            if (e == cudaSuccess) e = cudaMemsetAsync(E->cursor[s], 0, (size_t)E->T * 4, st);
            for (int p = 0; p < 2; p++)
                if (e == cudaSuccess) e = cudaMemsetAsync(E->bstart[p][s], 0, ((size_t)nbox + 1) * 8, st);
        }
        if (e == cudaSuccess) e = cudaMemsetAsync(E->d_cnt, 0, 4 * sizeof(long long), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(E->d_status, 0, sizeof(int), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(E->rhofx, 0, (size_t)maxint * 8, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(E->dacc, 0, (size_t)nbox * 16 * 8, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(E->dhist, 0, (size_t)nbox * TG_ENS_DIAG_CAP * 16 * 8, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(E->dcounter, 0, (size_t)nbox * 8, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) r = efail(E, TG_ERR_CUDA, "tg_ens_init: %s", cudaGetErrorString(e));
    }
    if (r) {
        snprintf(g_ens_error, sizeof g_ens_error, "%s", E->err);
        tg_ens_finalize(E);
        return r;
    }
    E->hf.assign((size_t)nbox * 9, nullptr);
    E->hp.assign(nbox, nullptr);
    E->hions.assign(nbox, nullptr);
    E->hlecs.assign(nbox, nullptr);
    for (int s = 0; s < 2; s++) E->hbstart[s].assign((size_t)nbox + 1, 0);
    *out = E;
    return TG_OK;
}

extern "C" void tg_ens_finalize(tg_ens *E) {
    if (!E) return;
    cudaSetDevice(E->device);
    if (E->st) cudaStreamSynchronize(E->st);
    {
        std::lock_guard<std::mutex> lock(g_const_mu);
        if (E->device >= 0 && E->device < TG_ENS_MAX_DEVICES && g_const_owner[E->device] == E)
            g_const_owner[E->device] = nullptr;
    }
    if (E->laps_done) cudaEventDestroy(E->laps_done);
    for (int p = 0; p < 2; p++)
        if (E->cycle[p]) cudaGraphExecDestroy(E->cycle[p]);
    for (void *q : E->allocs) cudaFree(q);
    for (int b = 0; b < 2; b++) {
        if (E->side[b]) cudaStreamDestroy(E->side[b]);
        if (E->join[b]) cudaEventDestroy(E->join[b]);
    }
    if (E->fork) cudaEventDestroy(E->fork);
    if (E->st) cudaStreamDestroy(E->st);
    delete E;
}

extern "C" const char *tg_ens_last_error(tg_ens *E) { return E ? E->err : g_ens_error; }

extern "C" int tg_ens_bind_fields(tg_ens *E, int32_t box, float *ex, float *ey, float *ez, float *bx, float *by,
                                  float *bz, float *curx, float *cury, float *curz) {
    if (!E) return TG_ERR_ARG;
    if (box < 0 || box >= E->nbox) return efail(E, TG_ERR_ARG, "tg_ens_bind_fields: box %d out of range", box);
    float *h[9] = {ex, ey, ez, bx, by, bz, curx, cury, curz};
    for (int a = 0; a < 9; a++) E->hf[(size_t)box * 9 + a] = h[a];
    return TG_OK;
}

extern "C" int tg_ens_bind_particles(tg_ens *E, int32_t box, void *p, int32_t *ions, int32_t *lecs) {
    if (!E) return TG_ERR_ARG;
    if (box < 0 || box >= E->nbox) return efail(E, TG_ERR_ARG, "tg_ens_bind_particles: box %d out of range", box);
    if (!p || !ions || !lecs) return efail(E, TG_ERR_ARG, "tg_ens_bind_particles: null argument");
    E->hp[box] = p;
    E->hions[box] = ions;
    E->hlecs[box] = lecs;
    return TG_OK;
}

static const size_t AOS = 40;

// work queue of the particle kernel: shape order 3 first, then by particles
// per tile, largest first (each box's tiles stay together)
static int build_work(tg_ens *E, const std::vector<long long> &nb) {
    std::vector<int> order(E->nbox);
    std::vector<double> cost(E->nbox);
    for (int b = 0; b < E->nbox; b++) {
        order[b] = b;
        cost[b] = (double)nb[b] / (double)E->g[b].ntiles;
    }
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        if (E->g[a].order != E->g[b].order) return E->g[a].order > E->g[b].order;
        return cost[a] > cost[b];
    });
    std::vector<int2> work;
    work.reserve(E->T);
    for (int o = 0; o < 3; o++) {
        E->nwork[o] = 0;
        E->wstart[o] = 0;
    }
    for (int b : order) {
        const int o = E->g[b].order - 1;
        if (E->nwork[o] == 0) E->wstart[o] = (int)work.size();
        for (int t = 0; t < E->g[b].ntiles; t++) work.push_back(make_int2(b, t));
        E->nwork[o] += E->g[b].ntiles;
    }
    ECK(cudaMemcpyAsync(E->d_work, work.data(), work.size() * sizeof(int2), cudaMemcpyHostToDevice, E->st));
    ECK(cudaStreamSynchronize(E->st));
    return TG_OK;
}

static int sort_species(tg_ens *E, int s, bool counted) {
    const int p = E->par;
    // a flat grid over the particles of every box
    const long long per = E->capacity / 256 + 1;
    const int grid = (int)(per < 152 * 16 ? per : 152 * 16);
    if (!counted) {
        k_ens_count<<<grid, 256, 0, E->st>>>(E->d_geom, E->sp[p][s], E->bstart[p][s], E->nbox, E->d_tofs,
                                             E->hist[s]);
        ECK(cudaGetLastError());
    }
    ECK(launch_scan(E->hist[s], E->tstart[s], E->cursor[s], E->T, E->d_cnt + 2 * (1 - p) + s, E->st));
    k_ens_bstart<<<1, 256, 0, E->st>>>(E->d_tofs, E->tstart[s], E->bstart[1 - p][s], E->nbox);
    ECK(cudaGetLastError());
    k_ens_scatter<<<grid, 256, 0, E->st>>>(E->d_geom, E->sp[p][s], E->sp[1 - p][s], E->bstart[p][s], E->nbox,
                                           E->d_tofs,
                                           E->tstart[s], E->cursor[s]);
    ECK(cudaGetLastError());
    return TG_OK;
}

static int sort_all(tg_ens *E, bool counted) {
    int r;
    if ((r = sort_species(E, 0, counted))) return r;
    if ((r = sort_species(E, 1, counted))) return r;
    E->par ^= 1;
    E->dirty = false;
    E->may_have_dead = false;
    return TG_OK;
}

static int ensure_sorted(tg_ens *E) {
    if (!E->dirty) return TG_OK;
    return sort_all(E, false);
}

extern "C" int tg_ens_sync_from_host(tg_ens *E, unsigned mask) {
    if (!E) return TG_ERR_ARG;
    const int groups[3][4] = {{0, 1, 2, (int)TG_SYNC_E}, {3, 4, 5, (int)TG_SYNC_B}, {6, 7, 8, (int)TG_SYNC_CUR}};
    for (int b = 0; b < E->nbox; b++)
        for (int gi = 0; gi < 3; gi++) {
            if (!(mask & (unsigned)groups[gi][3])) continue;
            for (int a = 0; a < 3; a++) {
                float *h = E->hf[(size_t)b * 9 + groups[gi][a]];
                if (!h)
                    return efail(E, TG_ERR_STATE, "tg_ens_sync_from_host: box %d field %d not bound", b,
                                 groups[gi][a]);
                ECK(cudaMemcpyAsync(E->f[groups[gi][a]] + E->fofs[b], h, (size_t)E->g[b].lot * 4,
                                    cudaMemcpyHostToDevice, E->st));
            }
        }
    if (mask & TG_SYNC_PARTICLES) {
        std::vector<long long> nb(E->nbox, 0);
        std::vector<long long> off[2];
        for (int s = 0; s < 2; s++) off[s].assign((size_t)E->nbox + 1, 0);
        for (int b = 0; b < E->nbox; b++) {
            if (!E->hp[b]) return efail(E, TG_ERR_STATE, "tg_ens_sync_from_host: box %d particles not bound", b);
            const long long n[2] = {*E->hions[b], *E->hlecs[b]};
            for (int s = 0; s < 2; s++) {
                if (n[s] < 0 || n[s] > E->cfg[b].maxhlf)
                    return efail(E, TG_ERR_OVERFLOW, "box %d species %d count %lld outside [0, maxhlf=%lld]", b, s,
                                 n[s], (long long)E->cfg[b].maxhlf);
                off[s][b + 1] = off[s][b] + n[s];
            }
            nb[b] = n[0] + n[1];
        }
        const int p = E->par;
        for (int b = 0; b < E->nbox; b++)
            for (int s = 0; s < 2; s++) {
                const long long n = off[s][b + 1] - off[s][b];
                if (n == 0) continue;
                const char *src = (const char *)E->hp[b] + (s == 0 ? 0 : (size_t)E->cfg[b].maxhlf * AOS);
                ECK(cudaMemcpyAsync(E->stage, src, (size_t)n * AOS, cudaMemcpyHostToDevice, E->st));
                ECK(launch_aos_to_soa(E->g[b], E->stage, sp_at(E->sp[p][s], off[s][b]), n, E->d_status, E->st));
            }
        for (int s = 0; s < 2; s++) {
            ECK(cudaMemcpyAsync(E->bstart[p][s], off[s].data(), ((size_t)E->nbox + 1) * 8, cudaMemcpyHostToDevice,
                                E->st));
            ECK(cudaMemcpyAsync(E->d_cnt + 2 * p + s, &off[s][E->nbox], 8, cudaMemcpyHostToDevice, E->st));
        }
        ECK(cudaStreamSynchronize(E->st));  // off[] lives on this stack frame
        int r = build_work(E, nb);
        if (r) return r;
        E->dirty = true;
        E->may_have_dead = true;
    }
    return TG_OK;
}

// box starts of the buffer in use (drops discarded particles first)
static int exact_starts(tg_ens *E) {
    if (E->may_have_dead || E->dirty) {
        int r = sort_all(E, false);
        if (r) return r;
    }
    for (int s = 0; s < 2; s++)
        ECK(cudaMemcpyAsync(E->hbstart[s].data(), E->bstart[E->par][s], ((size_t)E->nbox + 1) * 8,
                            cudaMemcpyDeviceToHost, E->st));
    ECK(cudaStreamSynchronize(E->st));
    return TG_OK;
}

extern "C" int tg_ens_sync_to_host(tg_ens *E, unsigned mask) {
    if (!E) return TG_ERR_ARG;
    const int groups[3][4] = {{0, 1, 2, (int)TG_SYNC_E}, {3, 4, 5, (int)TG_SYNC_B}, {6, 7, 8, (int)TG_SYNC_CUR}};
    for (int b = 0; b < E->nbox; b++)
        for (int gi = 0; gi < 3; gi++) {
            if (!(mask & (unsigned)groups[gi][3])) continue;
            for (int a = 0; a < 3; a++) {
                float *h = E->hf[(size_t)b * 9 + groups[gi][a]];
                if (!h)
                    return efail(E, TG_ERR_STATE, "tg_ens_sync_to_host: box %d field %d not bound", b,
                                 groups[gi][a]);
                ECK(cudaMemcpyAsync(h, E->f[groups[gi][a]] + E->fofs[b], (size_t)E->g[b].lot * 4,
                                    cudaMemcpyDeviceToHost, E->st));
            }
        }
    if (mask & TG_SYNC_PARTICLES) {
        int r = exact_starts(E);
        if (r) return r;
        for (int b = 0; b < E->nbox; b++) {
            if (!E->hp[b]) return efail(E, TG_ERR_STATE, "tg_ens_sync_to_host: box %d particles not bound", b);
            for (int s = 0; s < 2; s++) {
                const long long o = E->hbstart[s][b], n = E->hbstart[s][b + 1] - o;
                if (n > E->cfg[b].maxhlf)
                    return efail(E, TG_ERR_OVERFLOW, "box %d species %d holds %lld > maxhlf", b, s, n);
                if (n == 0) continue;
                ECK(launch_soa_to_aos(E->g[b], sp_at(E->sp[E->par][s], o), E->stage, n, E->st));
                char *dst = (char *)E->hp[b] + (s == 0 ? 0 : (size_t)E->cfg[b].maxhlf * AOS);
                ECK(cudaMemcpyAsync(dst, E->stage, (size_t)n * AOS, cudaMemcpyDeviceToHost, E->st));
            }
        }
    }
    ECK(cudaStreamSynchronize(E->st));
    if (mask & TG_SYNC_PARTICLES)
        for (int b = 0; b < E->nbox; b++) {
            *E->hions[b] = (int32_t)(E->hbstart[0][b + 1] - E->hbstart[0][b]);
            *E->hlecs[b] = (int32_t)(E->hbstart[1][b + 1] - E->hbstart[1][b]);
        }
    return check_status(E);
}

extern "C" int tg_ens_get_counts(tg_ens *E, int32_t box, int64_t *ions, int64_t *lecs) {
    if (!E || !ions || !lecs) return TG_ERR_ARG;
    if (box < 0 || box >= E->nbox) return efail(E, TG_ERR_ARG, "tg_ens_get_counts: box %d out of range", box);
    int r = exact_starts(E);
    if (r) return r;
    *ions = E->hbstart[0][box + 1] - E->hbstart[0][box];
    *lecs = E->hbstart[1][box + 1] - E->hbstart[1][box];
    return check_status(E);
}

// ---------------------------------------------------------------------------
// one lap of every box (order of tristanmainloop.F90:117-242, as the
// single-domain lap)
// ---------------------------------------------------------------------------
static int ens_lap(tg_ens *E, bool sort_now, int *nk) {
    cudaStream_t st = E->st;
    int k = 0;
    float **f9 = E->d_f9;
    const EnsBox *bx = E->d_box;
#define TG_EGHOST(A)                                                                                   \
    do {                                                                                               \
        k_ens_ghost<<<E->nblk[EK_GHOST], 256, 0, st>>>(bx, E->d_blk[EK_GHOST], E->f[A], E->f[A + 1],   \
                                                       E->f[A + 2]);                                   \
        ECK(cudaGetLastError());                                                                       \
        k++;                                                                                           \
    } while (0)
#define TG_EADV(KERN, KIND)                                                                            \
    do {                                                                                               \
        KERN<<<E->nblk[KIND], 256, 0, st>>>(bx, E->d_blk[KIND], f9);                                   \
        ECK(cudaGetLastError());                                                                       \
        k++;                                                                                           \
    } while (0)
    TG_EGHOST(3);
    TG_EGHOST(0);
    TG_EADV(k_ens_advance_b, EK_ADVB);
    TG_EGHOST(3);
    if (!E->fixed)
        for (int a = 6; a < 9; a++) ECK(cudaMemsetAsync(E->f[a], 0, (size_t)E->ncell * 4, st));
    ECK(cudaMemsetAsync(E->queue, 0, 3 * sizeof(int), st));
    const TileArgs *ta = E->d_targs + (size_t)(E->par * 2 + (sort_now ? 1 : 0)) * E->nbox;
    // shape order 3 on the lap's stream, orders 2 and 1 on two branches that
    // fill the SMs as the order-3 tiles drain
    // this lap's tile arguments into the constant-memory table
    if (E->use_const)
        ECK(cudaMemcpyToSymbolAsync(c_ens_targs, ta, (size_t)E->nbox * sizeof(TileArgs), 0, cudaMemcpyDeviceToDevice,
                                    st));
    ECK(cudaEventRecord(E->fork, st));
    for (int b = 0; b < 2; b++) ECK(cudaStreamWaitEvent(E->side[b], E->fork, 0));
    for (int o = 3; o >= 1; o--) {
        cudaStream_t so = o == 3 ? st : E->side[o == 2 ? 0 : 1];
        const int2 *w = E->d_work + E->wstart[o - 1];
        const int nw = E->nwork[o - 1];
        int *qu = E->queue + (o - 1);
        const int grid = E->tile_grid[o - 1];
        if (nw > 0 && E->use_const) {
            if (E->fixed) {
                if (o == 3) k_ens_tiles_c<3, true><<<grid, 256, E->smem, so>>>(w, nw, qu);
                else if (o == 2) k_ens_tiles_c<2, true><<<grid, 256, E->smem, so>>>(w, nw, qu);
                else k_ens_tiles_c<1, true><<<grid, 256, E->smem, so>>>(w, nw, qu);
            } else {
                if (o == 3) k_ens_tiles_c<3, false><<<grid, 256, E->smem, so>>>(w, nw, qu);
                else if (o == 2) k_ens_tiles_c<2, false><<<grid, 256, E->smem, so>>>(w, nw, qu);
                else k_ens_tiles_c<1, false><<<grid, 256, E->smem, so>>>(w, nw, qu);
            }
            ECK(cudaGetLastError());
            k++;
            continue;
        }
        if (nw > 0) {
            if (E->fixed) {
                if (o == 3) k_ens_tiles<3, true><<<grid, 256, E->smem, so>>>(ta, w, nw, qu);
                else if (o == 2) k_ens_tiles<2, true><<<grid, 256, E->smem, so>>>(ta, w, nw, qu);
                else k_ens_tiles<1, true><<<grid, 256, E->smem, so>>>(ta, w, nw, qu);
            } else {
                if (o == 3) k_ens_tiles<3, false><<<grid, 256, E->smem, so>>>(ta, w, nw, qu);
                else if (o == 2) k_ens_tiles<2, false><<<grid, 256, E->smem, so>>>(ta, w, nw, qu);
                else k_ens_tiles<1, false><<<grid, 256, E->smem, so>>>(ta, w, nw, qu);
            }
            ECK(cudaGetLastError());
            k++;
        }
    }
    for (int b = 0; b < 2; b++) {
        ECK(cudaEventRecord(E->join[b], E->side[b]));
        ECK(cudaStreamWaitEvent(st, E->join[b], 0));
    }
    TG_EADV(k_ens_advance_b, EK_ADVB);
    TG_EGHOST(3);
    TG_EADV(k_ens_advance_e, EK_ADVE);
    TG_EGHOST(0);
    if (E->fixed) {
        k_ens_fixed_to_float<<<E->nblk[EK_LOT], 256, 0, st>>>(bx, E->d_blk[EK_LOT], E->d_fx3, f9);
        ECK(cudaGetLastError());
        k++;
    }
    for (int axis = 0; axis < 2; axis++) {
        const int kind = axis == 0 ? EK_FOLD0 : EK_FOLD1;
        k_ens_fold<<<E->nblk[kind], 256, 0, st>>>(bx, E->d_blk[kind], axis, E->f[6], E->f[7], E->f[8]);
        ECK(cudaGetLastError());
        k++;
    }
    float *a3[3] = {E->f[6], E->f[7], E->f[8]};
    float *b3[3] = {E->ftmp[0], E->ftmp[1], E->ftmp[2]};
    for (int n = 0; n < E->ntimes; n++) {
        float *const *in = n % 2 == 0 ? a3 : b3;
        float *const *out = n % 2 == 0 ? b3 : a3;
        k_ens_filter<<<E->nblk[EK_LOT], 256, 0, st>>>(bx, E->d_blk[EK_LOT], in[0], in[1], in[2], out[0], out[1],
                                                      out[2]);
        ECK(cudaGetLastError());
        k++;
    }
    if (E->ntimes % 2 == 1)
        for (int cc = 0; cc < 3; cc++)
            ECK(cudaMemcpyAsync(a3[cc], b3[cc], (size_t)E->ncell * 4, cudaMemcpyDeviceToDevice, st));
    // add_current over the whole concatenated arrays (ghosts and padding
    // included; padding stays zero)
    Geom flat;
    memset(&flat, 0, sizeof flat);
    flat.lot = E->ncell;
    ECK(launch_add_current(flat, E->f, st));
    k++;
    if (sort_now) {
        int r = sort_all(E, true);
        if (r) return r;
        k += 6;
    }
#undef TG_EGHOST
#undef TG_EADV
    *nk = k;
    return TG_OK;
}

static int capture_cycle(tg_ens *E, int start_par) {
    const int se = E->sort_every;
    cudaGraph_t graph = nullptr;
    ECK(cudaStreamBeginCapture(E->st, cudaStreamCaptureModeThreadLocal));
    int r = TG_OK, nk = 0;
    for (int l = 0; l < 2 * se && r == TG_OK; l++) r = ens_lap(E, (l % se) == se - 1, &nk);
    cudaError_t e = cudaStreamEndCapture(E->st, &graph);
    if (r) {
        if (graph) cudaGraphDestroy(graph);
        return r;
    }
    if (e != cudaSuccess) return efail(E, TG_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&E->cycle[start_par], graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return efail(E, TG_ERR_CUDA, "graph instantiate failed: %s", cudaGetErrorString(e));
    E->kernels_per_step = nk;
    E->par = start_par;  // two sorts per cycle
    return TG_OK;
}

// called with g_const_mu held
static int claim_const_table(tg_ens *E) {
    tg_ens *&owner = g_const_owner[E->device];
    if (owner && owner != E) ECK(cudaStreamWaitEvent(E->st, owner->laps_done, 0));
    owner = E;
    return TG_OK;
}

static int ens_step_laps(tg_ens *E, int32_t nsteps);

extern "C" int tg_ens_step(tg_ens *E, int32_t nsteps) {
    if (!E || nsteps < 0) return TG_ERR_ARG;
    int r = ensure_sorted(E);
    if (r) return r;
    if (!E->use_const) return ens_step_laps(E, nsteps);
    // the laps are issued under the table's lock, so another ensemble that
    // steps next on this device waits for exactly these laps
    std::lock_guard<std::mutex> lock(g_const_mu);
    if ((r = claim_const_table(E))) return r;
    if ((r = ens_step_laps(E, nsteps))) return r;
    ECK(cudaEventRecord(E->laps_done, E->st));
    return TG_OK;
}

static int ens_step_laps(tg_ens *E, int32_t nsteps) {
    int r = TG_OK;
    if (nsteps > 0) E->may_have_dead = true;
    const int se = E->sort_every, cyc = 2 * se;
    int left = nsteps;
    while (left > 0) {
        const int phase = (int)(E->lap % cyc);
        if (phase == 0 && left >= cyc) {
            const int p = E->par;
            if (!E->cycle[p] && (r = capture_cycle(E, p))) return r;
            ECK(cudaGraphLaunch(E->cycle[p], E->st));
            E->lap += cyc;
            left -= cyc;
        } else {
            int nk = 0;
            if ((r = ens_lap(E, (phase % se) == se - 1, &nk))) return r;
            E->kernels_per_step = nk;
            E->lap += 1;
            left -= 1;
        }
    }
    return TG_OK;
}

extern "C" int tg_ens_step_timed(tg_ens *E, int32_t nsteps, float *ms) {
    if (!E || !ms) return TG_ERR_ARG;
    int r = ensure_sorted(E);
    if (r) return r;
    cudaEvent_t a, b;
    ECK(cudaEventCreate(&a));
    ECK(cudaEventCreate(&b));
    ECK(cudaEventRecord(a, E->st));
    r = tg_ens_step(E, nsteps);
    ECK(cudaEventRecord(b, E->st));
    ECK(cudaEventSynchronize(b));
    ECK(cudaEventElapsedTime(ms, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (r) return r;
    return check_status(E);
}

extern "C" int tg_ens_synchronize(tg_ens *E) {
    if (!E) return TG_ERR_ARG;
    ECK(cudaStreamSynchronize(E->st));
    return check_status(E);
}

extern "C" int32_t tg_ens_kernels_per_step(tg_ens *E) { return E ? E->kernels_per_step : 0; }

extern "C" int tg_ens_diag_fp64(tg_ens *E, int32_t box, tg_diag *out) {
    if (!E || !out) return TG_ERR_ARG;
    if (box < 0 || box >= E->nbox) return efail(E, TG_ERR_ARG, "tg_ens_diag_fp64: box %d out of range", box);
    int r = ensure_sorted(E);
    if (r) return r;
    const long long o = E->fofs[box];
    DiagLaunch d;
    memset(&d, 0, sizeof d);
    d.g = E->g[box];
    d.P = E->P[box];
    for (int s = 0; s < 2; s++) {
        d.sp[s] = E->sp[E->par][s];
        d.tstart[s] = E->tstart[s] + E->tofs[box];
        d.mass[s] = fabsf(E->P[box].qs[s] / E->P[box].qm[s]);
    }
    for (int a = 0; a < 6; a++) d.f[a] = E->f[a] + o;
    d.rhofx = E->rhofx;
    d.rho[0] = E->rho[0];
    d.rho[1] = E->rho[1];
    d.acc = E->dacc + (size_t)box * 16;
    d.hist = E->dhist + (size_t)box * TG_ENS_DIAG_CAP * 16;
    d.hist_cap = TG_ENS_DIAG_CAP;
    d.counter = E->dcounter + box;
    d.ntimes = E->ntimes;
    d.status = E->d_status;
    d.particles = true;
    ECK(launch_diag(d, E->st));
    unsigned long long cnt = 0;
    ECK(cudaMemcpyAsync(&cnt, E->dcounter + box, 8, cudaMemcpyDeviceToHost, E->st));
    ECK(cudaStreamSynchronize(E->st));
    double h[16];
    const unsigned long long slot = (cnt - 1ull) % (unsigned long long)TG_ENS_DIAG_CAP;
    ECK(cudaMemcpyAsync(h, d.hist + slot * 16, 16 * 8, cudaMemcpyDeviceToHost, E->st));
    ECK(cudaStreamSynchronize(E->st));
    record_to_diag(h, out);
    return check_status(E);
}

// ---------------------------------------------------------------------------
// autotuner: one tile shape and re-sort cadence for all boxes, chosen by
// timing short runs of the batched lap on the given boxes
// ---------------------------------------------------------------------------
extern "C" int tg_ens_autotune(tg_config *cfgs, int32_t nbox, void *const *p, int32_t *const *ions,
                               int32_t *const *lecs, int32_t laps, float *best_ms, float *table,
                               int32_t table_len) {
    if (!cfgs || !p || !ions || !lecs || nbox < 1 || laps < 1) return -TG_ERR_ARG;
    struct Cand {
        int tx, ty, se;
    };
    std::vector<Cand> cands;
    const int tiles[5][2] = {{16, 16}, {32, 16}, {16, 32}, {32, 32}, {8, 8}};
    for (auto &t : tiles)
        for (int se = 1; se <= 3; se++) cands.push_back({t[0], t[1], se});
    float best = 1e30f;
    Cand bestc = cands[0];
    int row = 0;
    std::vector<tg_config> c(cfgs, cfgs + nbox);
    std::vector<int32_t> ni(nbox), nl(nbox);
    for (const Cand &cd : cands) {
        for (int b = 0; b < nbox; b++) {
            c[b].tile[0] = cd.tx;
            c[b].tile[1] = cd.ty;
            c[b].tile[2] = 1;
            c[b].sort_every = cd.se;
            ni[b] = *ions[b];
            nl[b] = *lecs[b];
        }
        tg_ens *E = nullptr;
        float ms = -1.0f;
        if (tg_ens_init(c.data(), nbox, &E) == TG_OK) {
            int r = TG_OK;
            for (int b = 0; b < nbox && !r; b++) r = tg_ens_bind_particles(E, b, p[b], &ni[b], &nl[b]);
            if (!r && tg_ens_sync_from_host(E, TG_SYNC_PARTICLES) == TG_OK && tg_ens_step(E, 2 * cd.se) == TG_OK &&
                tg_ens_synchronize(E) == TG_OK && tg_ens_step_timed(E, laps * 2 * cd.se, &ms) == TG_OK) {
                ms /= (float)(laps * 2 * cd.se);
                if (ms < best) {
                    best = ms;
                    bestc = cd;
                }
            } else {
                ms = -1.0f;
            }
            tg_ens_finalize(E);
        }
        if (table && row < table_len) {
            table[5 * row + 0] = (float)cd.tx;
            table[5 * row + 1] = (float)cd.ty;
            table[5 * row + 2] = 1.0f;
            table[5 * row + 3] = (float)cd.se;
            table[5 * row + 4] = ms;
            row++;
        }
    }
    if (best >= 1e30f) return -TG_ERR_STATE;
    for (int b = 0; b < nbox; b++) {
        cfgs[b].tile[0] = bestc.tx;
        cfgs[b].tile[1] = bestc.ty;
        cfgs[b].tile[2] = 1;
        cfgs[b].sort_every = bestc.se;
    }
    if (best_ms) *best_ms = best;
    return row;
}

// Field kernels of the GB300 TRISTAN-MP hot path (sm_103a).
//
// All arrays keep the reference's Fortran layout (mx,my,mz), x fastest, so a
// warp reads 32 consecutive x cells (coalesced 128-byte lines). Each kernel
// is one pass over its cells and is HBM-bound; the stencils round exactly as
// the reference (compiled without FMA contraction).
#include <cuda_runtime.h>

#include "tg_fields.cuh"

namespace tg {

static inline int blocks_for(long long n, int bs) {
    long long b = (n + bs - 1) / bs;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;
    return (int)b;
}

__global__ void k_ghost(Geom g, float *a, float *b, float *c, GhostAxis ax, GhostAxis ay, GhostAxis az,
                        long long nX, long long nY, long long nZ) {
    const long long total = nX + nY + nZ;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x)
        ghost_one(g, a, b, c, ax, ay, az, nX, nY, t);
}

cudaError_t launch_ghost(const Geom &g, float *a, float *b, float *c, GhostKind kind, cudaStream_t st) {
    GhostAxis ax[3];
    long long n[3];
    ghost_plan(g, kind, ax, n);
    const long long total = n[0] + n[1] + n[2];
    if (total == 0) return cudaSuccess;
    k_ghost<<<blocks_for(total, 256), 256, 0, st>>>(g, a, b, c, ax[0], ax[1], ax[2], n[0], n[1], n[2]);
    return cudaGetLastError();
}

template <int DIM>
__global__ void k_advance_b(Geom g, Box bx_, float cst, const float *__restrict__ ex, const float *__restrict__ ey,
                            const float *__restrict__ ez, float *bx, float *by, float *bz) {
    const long long total = (long long)bx_.ni * bx_.nj * bx_.nk;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x)
        advance_b_one<DIM>(g, bx_, cst, ex, ey, ez, bx, by, bz, t);
}

template <int DIM>
__global__ void k_advance_e(Geom g, Box b_, float cst, float *ex, float *ey, float *ez, const float *__restrict__ bx,
                            const float *__restrict__ by, const float *__restrict__ bz) {
    const long long total = (long long)b_.ni * b_.nj * b_.nk;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x)
        advance_e_one<DIM>(g, b_, cst, ex, ey, ez, bx, by, bz, t);
}

cudaError_t launch_advance_b(const Geom &g, const Params &P, float *const *f, cudaStream_t st) {
    Box b;
    int i2, j2, k2;
    b_range(g, 0, b.i1, i2);
    b_range(g, 1, b.j1, j2);
    b_range(g, 2, b.k1, k2);
    b.ni = i2 - b.i1 + 1;
    b.nj = j2 - b.j1 + 1;
    b.nk = k2 - b.k1 + 1;
    const float cst = P.corr * (0.5f * P.c);
    const long long n = (long long)b.ni * b.nj * b.nk;
    if (g.dims == 3) k_advance_b<3><<<blocks_for(n, 256), 256, 0, st>>>(g, b, cst, f[0], f[1], f[2], f[3], f[4], f[5]);
    else k_advance_b<2><<<blocks_for(n, 256), 256, 0, st>>>(g, b, cst, f[0], f[1], f[2], f[3], f[4], f[5]);
    return cudaGetLastError();
}

cudaError_t launch_advance_e(const Geom &g, const Params &P, float *const *f, cudaStream_t st) {
    Box b;
    int i2, j2, k2;
    e_range(g, 0, b.i1, i2);
    e_range(g, 1, b.j1, j2);
    e_range(g, 2, b.k1, k2);
    b.ni = i2 - b.i1 + 1;
    b.nj = j2 - b.j1 + 1;
    b.nk = k2 - b.k1 + 1;
    const float cst = P.corr * P.c;
    const long long n = (long long)b.ni * b.nj * b.nk;
    if (g.dims == 3) k_advance_e<3><<<blocks_for(n, 256), 256, 0, st>>>(g, b, cst, f[0], f[1], f[2], f[3], f[4], f[5]);
    else k_advance_e<2><<<blocks_for(n, 256), 256, 0, st>>>(g, b, cst, f[0], f[1], f[2], f[3], f[4], f[5]);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// add_current (code/fields.F90:1372-1395), float4 vectorised over the array
// ---------------------------------------------------------------------------
__global__ void k_add_current(long long n, float *ex, float *ey, float *ez, const float *__restrict__ cx,
                              const float *__restrict__ cy, const float *__restrict__ cz) {
    const long long n4 = n / 4;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n4;
         t += (long long)gridDim.x * blockDim.x) {
        float4 e = reinterpret_cast<float4 *>(ex)[t];
        float4 c = reinterpret_cast<const float4 *>(cx)[t];
        e.x = e.x + c.x; e.y = e.y + c.y; e.z = e.z + c.z; e.w = e.w + c.w;
        reinterpret_cast<float4 *>(ex)[t] = e;
        e = reinterpret_cast<float4 *>(ey)[t];
        c = reinterpret_cast<const float4 *>(cy)[t];
        e.x = e.x + c.x; e.y = e.y + c.y; e.z = e.z + c.z; e.w = e.w + c.w;
        reinterpret_cast<float4 *>(ey)[t] = e;
        e = reinterpret_cast<float4 *>(ez)[t];
        c = reinterpret_cast<const float4 *>(cz)[t];
        e.x = e.x + c.x; e.y = e.y + c.y; e.z = e.z + c.z; e.w = e.w + c.w;
        reinterpret_cast<float4 *>(ez)[t] = e;
    }
    // tail
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t < n - 4 * n4) {
        const long long l = 4 * n4 + t;
        ex[l] = ex[l] + cx[l];
        ey[l] = ey[l] + cy[l];
        ez[l] = ez[l] + cz[l];
    }
}

cudaError_t launch_add_current(const Geom &g, float *const *f, cudaStream_t st) {
    k_add_current<<<blocks_for(g.lot / 4 + 1, 256), 256, 0, st>>>(g.lot, f[0], f[1], f[2], f[6], f[7], f[8]);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// exchange_current for one rank (code/fieldboundaries.F90:1768-2189):
// per axis, cur(ng/2+1..ng) += cur(m-ng/2..m), then
// cur(m-(ng-1)..m-(ng/2+1)) += cur(1..ng/2). Axis order x, y, z. One
// thread per target cell; an axis with at least nghost interior cells has
// disjoint target slabs and folds in one launch, a thinner one in two
// ordered launches (slab 1, then slab 2), as the reference adds them.
// ---------------------------------------------------------------------------
__global__ void k_fold(Geom g, int axis, int m, int ng, float *cx, float *cy, float *cz, int q5, int slab) {
    const long long total = fold_cells(g, axis, slab);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x)
        fold_one(g, axis, m, ng, cx, cy, cz, q5, t, slab);
}

cudaError_t launch_fold(const Geom &g, const Params &P, float *const *cur, cudaStream_t st) {
    for (int axis = 0; axis < 3; axis++) {
        if (axis == 2 && g.dims == 2) break;
        if (!g.per[axis]) continue;
        const int m = axis == 0 ? g.mx : axis == 1 ? g.my : g.mz;
        const int ng = axis == 2 ? g.ngz : g.ng;
        const int q5 = (axis == 1) && (P.quirks & TG_QUIRK_Q5_LHS);
        const bool one = fold_in_one_pass(g, axis);
        for (int slab = one ? -1 : 0; slab < (one ? 0 : 2); slab++) {
            const long long total = fold_cells(g, axis, slab);
            k_fold<<<blocks_for(total, 256), 256, 0, st>>>(g, axis, m, ng, cur[0], cur[1], cur[2], q5, slab);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

int fold_launches(const Geom &g) {
    int n = 0;
    for (int axis = 0; axis < g.dims; axis++)
        if (g.per[axis]) n += fold_in_one_pass(g, axis) ? 1 : 2;
    return n;
}

template <int DIM>
__global__ void __launch_bounds__(256) k_filter(Geom g, const float *__restrict__ i0, const float *__restrict__ i1,
                                                const float *__restrict__ i2, float *o0, float *o1, float *o2) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.lot;
         t += (long long)gridDim.x * blockDim.x)
        filter_one<DIM>(g, i0, i1, i2, o0, o1, o2, t);
}

// 3D pass staged through shared memory: a CTA owns a 32 x 8 column of
// cells and marches up TG_F3_KC planes, keeping the refreshed input planes
// k-1, k, k+1 (with a one-cell halo) of all three components in a ring, so
// every input element is read from HBM about once per pass instead of 27
// times through the cache. The plane k+2 is loaded into registers before
// plane k is filtered and stored into the ring after it, so its memory
// latency overlaps the stencil work. Each thread filters two neighbouring
// x cells: a row's four values come in two 8-byte shared loads and serve
// both cells' stencils (the 27 terms of each cell three times fewer shared
// loads than one cell per thread); each cell runs the same selection and
// the same stencil27 as filter_one.
#define TG_F3_CX 32  // cells per CTA along x (two per thread)
#define TG_F3_NX 16  // threads per CTA along x
#define TG_F3_TY 8
#define TG_F3_KC 32
#define TG_F3_NT (TG_F3_NX * TG_F3_TY)
#define TG_F3_SX (TG_F3_CX + 2)
#define TG_F3_SY (TG_F3_TY + 2)
#define TG_F3_PER ((TG_F3_SX * TG_F3_SY + TG_F3_NT - 1) / TG_F3_NT)  // halo cells per thread
__global__ void __launch_bounds__(TG_F3_NT)
    k_filter3d(Geom g, const float *__restrict__ i0, const float *__restrict__ i1, const float *__restrict__ i2,
               float *o0, float *o1, float *o2) {
    constexpr int SX = TG_F3_SX, SY = TG_F3_SY, PER = TG_F3_PER;
    // [component][plane ring][y][x]; rows of 34 floats keep every even x
    // 8-byte aligned
    __shared__ __align__(16) float sm[3][3][SY][SX];
    const RefreshMap Rx{g.mx, g.ng, g.per[0]}, Ry{g.my, g.ng, g.per[1]}, Rz{g.mz, g.ngz, g.per[2]};
    const int ib = blockIdx.x * TG_F3_CX + 1, jb = blockIdx.y * TG_F3_TY + 1;
    const int kb = blockIdx.z * TG_F3_KC + 1;
    const int ke = min(kb + TG_F3_KC, g.mz + 1);
    const int tid = threadIdx.y * TG_F3_NX + threadIdx.x;
    // this thread's halo cells of a plane: their (refreshed) x-y offset, or
    // -1 outside the array; each plane adds its (refreshed) z offset
    long long xy[PER];
    int slot_xy[PER];
#pragma unroll
    for (int e = 0; e < PER; e++) {
        const int t = tid + e * TG_F3_NT;
        slot_xy[e] = t < SX * SY ? t : -1;
        xy[e] = -1;
        if (t < SX * SY) {
            const int i = ib - 1 + t % SX, j = jb - 1 + t / SX;
            if (i >= 1 && i <= g.mx && j >= 1 && j <= g.my) xy[e] = lin(g, Rx(i), Ry(j), 1);
        }
    }
    float stage[3][PER];
    auto fetch = [&](int k) {  // plane k into registers
        const bool kin = k >= 1 && k <= g.mz;
        const long long zo = kin ? g.sz * (long long)(Rz(k) - 1) : 0;
#pragma unroll
        for (int e = 0; e < PER; e++) {
            const bool ok = kin && xy[e] >= 0;
            stage[0][e] = ok ? i0[xy[e] + zo] : 0.0f;
            stage[1][e] = ok ? i1[xy[e] + zo] : 0.0f;
            stage[2][e] = ok ? i2[xy[e] + zo] : 0.0f;
        }
    };
    auto put = [&](int k) {  // registers into plane k's ring slot
        const int slot = (k + 3) % 3;
#pragma unroll
        for (int e = 0; e < PER; e++)
            if (slot_xy[e] >= 0) {
                const int lx = slot_xy[e] % SX, ly = slot_xy[e] / SX;
#pragma unroll
                for (int c = 0; c < 3; c++) sm[c][slot][ly][lx] = stage[c][e];
            }
    };
    const int ilo = g.ng / 2 + 1, ihi = g.mx - (g.ng / 2 + 1);
    const int jlo = g.ng / 2 + 1, jhi = g.my - (g.ng / 2 + 1);
    const int klo = g.ngz / 2 + 1, khi = g.mz - (g.ngz / 2 + 1);
    const int ia = ib + 2 * threadIdx.x, j = jb + threadIdx.y;  // cells ia and ia + 1
    const int lx = 2 * threadIdx.x, ly = threadIdx.y + 1;       // slot of x = ia - 1
    fetch(kb - 1);
    put(kb - 1);
    fetch(kb);
    put(kb);
    fetch(kb + 1);
    put(kb + 1);
    __syncthreads();
    for (int k = kb; k < ke; k++) {
        if (k + 1 < ke) fetch(k + 2);  // in flight while plane k is filtered
        if (ia <= g.mx && j <= g.my) {
            const bool kin = k >= klo && k <= khi;
            const bool jxy = j >= jlo && j <= jhi, jz = j >= jlo && j <= jhi + 2;
            const bool ina = kin && ia >= ilo && ia <= ihi, inb = kin && ia + 1 >= ilo && ia + 1 <= ihi;
            const int sl[3] = {(k + 2) % 3, k % 3, (k + 1) % 3};
            float ra[3], rb[3];
#pragma unroll
            for (int c = 0; c < 3; c++) {
                const bool jc = c == 2 ? jz : jxy;
                // rows (dj, dk): x = ia - 1 .. ia + 2
                float r[3][3][4];
#pragma unroll
                for (int dk = 0; dk < 3; dk++)
#pragma unroll
                    for (int dj = 0; dj < 3; dj++) {
                        const float2 p = *reinterpret_cast<const float2 *>(&sm[c][sl[dk]][ly + dj - 1][lx]);
                        const float2 q = *reinterpret_cast<const float2 *>(&sm[c][sl[dk]][ly + dj - 1][lx + 2]);
                        r[dk][dj][0] = p.x;
                        r[dk][dj][1] = p.y;
                        r[dk][dj][2] = q.x;
                        r[dk][dj][3] = q.y;
                    }
                ra[c] = (jc && ina) ? stencil27([&](int di, int dj, int dk) { return r[dk + 1][dj + 1][di + 1]; })
                                    : r[1][1][1];
                rb[c] = (jc && inb) ? stencil27([&](int di, int dj, int dk) { return r[dk + 1][dj + 1][di + 2]; })
                                    : r[1][1][2];
            }
            const long long t = lin(g, ia, j, k);
            o0[t] = ra[0];
            o1[t] = ra[1];
            o2[t] = ra[2];
            if (ia + 1 <= g.mx) {
                o0[t + 1] = rb[0];
                o1[t + 1] = rb[1];
                o2[t + 1] = rb[2];
            }
        }
        __syncthreads();  // plane k-1's slot is free
        if (k + 1 < ke) {
            put(k + 2);
            __syncthreads();
        }
    }
}

cudaError_t launch_filter_pass(const Geom &g, float *const *in, float *const *out, cudaStream_t st) {
    if (g.dims == 3) {
        const dim3 grid((g.mx + TG_F3_CX - 1) / TG_F3_CX, (g.my + TG_F3_TY - 1) / TG_F3_TY,
                        (g.mz + TG_F3_KC - 1) / TG_F3_KC);
        k_filter3d<<<grid, dim3(TG_F3_NX, TG_F3_TY), 0, st>>>(g, in[0], in[1], in[2], out[0], out[1], out[2]);
    } else {
        k_filter<2><<<blocks_for(g.lot, 256), 256, 0, st>>>(g, in[0], in[1], in[2], out[0], out[1], out[2]);
    }
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Primal-averaged copies for the 3D gather (code/particles_movedeposit.F90:
// 395-404): cshift(.,-1) wraps over the whole local array.
// ---------------------------------------------------------------------------
__global__ void k_primal(Geom g, const float *__restrict__ ex, const float *__restrict__ ey,
                         const float *__restrict__ ez, const float *__restrict__ bx, const float *__restrict__ by,
                         const float *__restrict__ bz, float4 *prim) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.lot;
         t += (long long)gridDim.x * blockDim.x) {
        const int ti = (int)t;  // fewer than 2^31 cells
        const int i = ti % g.mx + 1;
        const int r = ti / g.mx;
        const int j = r % g.my + 1;
        const int k = r / g.my + 1;
        const int im = i == 1 ? g.mx : i - 1, jm = j == 1 ? g.my : j - 1, km = k == 1 ? g.mz : k - 1;
        const long long lxm = lin(g, im, j, k), lym = lin(g, i, jm, k), lzm = lin(g, i, j, km);
        prim[2 * t] = make_float4(0.5f * (ex[t] + ex[lxm]), 0.5f * (ey[t] + ey[lym]), 0.5f * (ez[t] + ez[lzm]),
                                  0.5f * (bx[t] + bx[lym]));
        prim[2 * t + 1] = make_float4(0.5f * (by[t] + by[lxm]),
                                      0.5f * (0.5f * (bz[t] + bz[lxm]) + 0.5f * (bz[lym] + bz[lin(g, im, jm, k)])),
                                      0.0f, 0.0f);
    }
}

cudaError_t launch_primal(const Geom &g, float *const *f, float4 *prim, cudaStream_t st) {
    k_primal<<<blocks_for(g.lot, 256), 256, 0, st>>>(g, f[0], f[1], f[2], f[3], f[4], f[5], prim);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// int64 fixed-point accumulators -> float currents; clears the accumulators
// ---------------------------------------------------------------------------
__global__ void k_fixed_to_float(long long n, double inv, unsigned long long *f0, unsigned long long *f1,
                                 unsigned long long *f2, float *c0, float *c1, float *c2) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        fixed_to_float_one(inv, f0, f1, f2, c0, c1, c2, t);
}

cudaError_t launch_fixed_to_float(const Geom &g, const Params &P, unsigned long long *const *fx, float *const *cur,
                                  cudaStream_t st) {
    k_fixed_to_float<<<blocks_for(g.lot, 256), 256, 0, st>>>(g.lot, P.fx_inv, fx[0], fx[1], fx[2], cur[0], cur[1],
                                                             cur[2]);
    return cudaGetLastError();
}

}  // namespace tg

// Per-cell bodies of the field kernels of the GB300 TRISTAN-MP hot path.
// The single-domain kernels (tg_fields.cu) and the box-batched ensemble
// kernels (tg_ensemble.cu) run the same function for each cell, so both give
// the same bits.
#pragma once

#include "tg_internal.cuh"

namespace tg {

// ---------------------------------------------------------------------------
// Ghost layers. bc_b1 / bc_e1 (code/fieldboundaries.F90:181-392) copy
// nghost/2 layers per side, axis by axis (x, then y over the x-filled
// layers, then z); the filter's refresh (code/filter.F90:71-98) copies one
// layer per side. Composed, every written cell receives the value of the
// cell W(i),W(j),W(k) with W the per-axis periodic image of the written
// layers (identity elsewhere, layer m is never written); that source is
// never itself written, so one gather pass over the ghost shell gives the
// sequential result.
// ---------------------------------------------------------------------------
struct GhostAxis {
    int m, ng, per, nt;  // extent, ghost width, periodic, number of target layers
    int kind;
    __device__ int target(int r) const {
        if (kind == GHOST_BC) return r < ng / 2 ? r + 1 : m - ng / 2 + (r - ng / 2);
        return r == 0 ? ng / 2 : m - ng / 2;
    }
    __device__ int nontarget(int r) const {
        if (nt == 0) return r + 1;
        if (kind == GHOST_BC) return r < m - ng ? ng / 2 + 1 + r : m;
        int l = r + 1;
        if (l >= ng / 2) l++;
        if (l >= m - ng / 2) l++;
        return l;
    }
    __device__ int image(int t) const {
        if (nt == 0) return t;
        const int P = m - ng;
        if (kind == GHOST_BC) {
            if (t <= ng / 2) return t + P;
            if (t >= m - ng / 2 && t <= m - 1) return t - P;
            return t;
        }
        if (t == ng / 2) return t + P;
        if (t == m - ng / 2) return t - P;
        return t;
    }
};

__host__ __device__ inline int ghost_targets(int per, int kind, int ng, bool active) {
    if (!per || !active) return 0;
    return kind == GHOST_BC ? ng - 1 : 2;
}

// the three gather axes of one ghost pass and its cells per part (x-target
// layers; y-target layers over the x non-targets; z-target layers)
inline void ghost_plan(const Geom &g, GhostKind kind, GhostAxis ax[3], long long n[3]) {
    ax[0] = GhostAxis{g.mx, g.ng, g.per[0], ghost_targets(g.per[0], kind, g.ng, true), kind};
    ax[1] = GhostAxis{g.my, g.ng, g.per[1], ghost_targets(g.per[1], kind, g.ng, true), kind};
    ax[2] = GhostAxis{g.mz, g.ngz, g.per[2], ghost_targets(g.per[2], kind, g.ngz, g.dims == 3), kind};
    n[0] = (long long)ax[0].nt * g.my * g.mz;
    n[1] = (long long)(g.mx - ax[0].nt) * ax[1].nt * g.mz;
    n[2] = (long long)(g.mx - ax[0].nt) * (g.my - ax[1].nt) * ax[2].nt;
}

__device__ __forceinline__ void ghost_one(const Geom &g, float *a, float *b, float *c, const GhostAxis &ax,
                                          const GhostAxis &ay, const GhostAxis &az, long long nX, long long nY,
                                          long long t) {
    // 32-bit index arithmetic: the ghost shell holds fewer than 2^31 cells
    int i, j, k;
    if (t < nX) {  // x-target layers, every j, k
        int r = (int)t;
        i = ax.target(r % ax.nt);
        r /= ax.nt;
        j = r % g.my + 1;
        k = r / g.my + 1;
    } else if (t < nX + nY) {  // x non-target, y-target, every k
        int r = (int)(t - nX);
        const int nnx = g.mx - ax.nt;
        i = ax.nontarget(r % nnx);
        r /= nnx;
        j = ay.target(r % ay.nt);
        k = r / ay.nt + 1;
    } else {  // x, y non-target, z-target
        int r = (int)(t - nX - nY);
        const int nnx = g.mx - ax.nt, nny = g.my - ay.nt;
        i = ax.nontarget(r % nnx);
        r /= nnx;
        j = ay.nontarget(r % nny);
        k = az.target(r / nny);
    }
    const long long dst = lin(g, i, j, k);
    const long long src = lin(g, ax.image(i), ay.image(j), az.image(k));
    a[dst] = a[src];
    b[dst] = b[src];
    c[dst] = c[src];
}

// ---------------------------------------------------------------------------
// Update ranges of advance_b_halfstep / advance_e_fullstep for one rank
// (code/fields.F90:593-665, :746-821).
// ---------------------------------------------------------------------------
inline void b_range(const Geom &g, int axis, int &a1, int &a2) {
    const int m = axis == 0 ? g.mx : axis == 1 ? g.my : g.mz;
    const int ng = axis == 2 ? g.ngz : g.ng;
    if (axis == 2 && g.dims == 2) { a1 = 1; a2 = 1; return; }
    if (g.per[axis]) { a1 = ng / 2 + 1; a2 = m - (ng / 2 + 1); }
    else { a1 = 1; a2 = m - 1; }
}

inline void e_range(const Geom &g, int axis, int &a1, int &a2) {
    const int m = axis == 0 ? g.mx : axis == 1 ? g.my : g.mz;
    const int ng = axis == 2 ? g.ngz : g.ng;
    if (axis == 2) {
        if (g.dims == 2) { a1 = 1; a2 = 1; return; }
        a1 = ng / 2;  // fields.F90:818-819 forces the full z range (Q7)
        a2 = m;
        return;
    }
    if (g.per[axis]) { a1 = ng / 2 + 1; a2 = m - (ng / 2 + 1); }
    else { a1 = ng / 2; a2 = m; }
}

struct Box {
    int i1, j1, k1, ni, nj, nk;
};

template <int DIM>
__device__ __forceinline__ void advance_b_one(const Geom &g, const Box &bx_, float cst, const float *__restrict__ ex,
                                              const float *__restrict__ ey, const float *__restrict__ ez, float *bx,
                                              float *by, float *bz, long long t) {
    // 32-bit index arithmetic: a box holds fewer than 2^31 cells
    const int ti = (int)t;
    const int i = ti % bx_.ni + bx_.i1;
    const int r = ti / bx_.ni;
    const int j = r % bx_.nj + bx_.j1;
    const int k = r / bx_.nj + bx_.k1;
    const long long l = lin(g, i, j, k);
    const long long lx = l + 1, ly = l + g.sy;
    if (DIM == 3) {
        const long long lz = l + g.sz;
        bx[l] = bx[l] + cst * (ey[lz] - ey[l] - ez[ly] + ez[l]);
        by[l] = by[l] + cst * (ez[lx] - ez[l] - ex[lz] + ex[l]);
        bz[l] = bz[l] + cst * (ex[ly] - ex[l] - ey[lx] + ey[l]);
    } else {
        bx[l] = bx[l] + cst * (-ez[ly] + ez[l]);
        by[l] = by[l] + cst * (ez[lx] - ez[l]);
        bz[l] = bz[l] + cst * (ex[ly] - ex[l] - ey[lx] + ey[l]);
    }
}

template <int DIM>
__device__ __forceinline__ void advance_e_one(const Geom &g, const Box &b_, float cst, float *ex, float *ey, float *ez,
                                              const float *__restrict__ bx, const float *__restrict__ by,
                                              const float *__restrict__ bz, long long t) {
    const int ti = (int)t;
    const int i = ti % b_.ni + b_.i1;
    const int r = ti / b_.ni;
    const int j = r % b_.nj + b_.j1;
    const int k = r / b_.nj + b_.k1;
    const long long l = lin(g, i, j, k);
    const long long lx = l - 1, ly = l - g.sy;
    if (DIM == 3) {
        const long long lz = l - g.sz;
        ex[l] = ex[l] + cst * (by[lz] - by[l] - bz[ly] + bz[l]);
        ey[l] = ey[l] + cst * (bz[lx] - bz[l] - bx[lz] + bx[l]);
        ez[l] = ez[l] + cst * (bx[ly] - bx[l] - by[lx] + by[l]);
    } else {
        ex[l] = ex[l] + cst * (-bz[ly] + bz[l]);
        ey[l] = ey[l] + cst * (bz[lx] - bz[l]);
        ez[l] = ez[l] + cst * (bx[ly] - bx[l] - by[lx] + by[l]);
    }
}

// One target cell of the current fold of one axis. The reference snapshots
// both source slabs first, then adds slab 1 (cur(ng/2+1 : ng) +=
// cur(m-ng/2 : m)) and after it slab 2 (cur(m-(ng-1) : m-(ng/2+1)) +=
// cur(1 : ng/2)) (code/fieldboundaries.F90:1797-1812). slab < 0 covers
// both slabs in one index range (t < nb1 faces: slab 1), for grids whose
// two target ranges are disjoint; slab 0 / 1 index one slab alone, for the
// ordered two-launch form.
__device__ __forceinline__ void fold_one(const Geom &g, int axis, int m, int ng, float *cx, float *cy, float *cz,
                                         int q5, long long t, int slab = -1) {
    const int nb1 = ng / 2 + 1;
    const int n1 = axis == 0 ? g.my : g.mx;  // first face extent
    const int n2 = axis == 2 ? g.my : g.mz;  // second face extent
    const int face = n1 * n2, ti = (int)t;
    const int layer = ti / face + (slab == 1 ? nb1 : 0);
    const int f = ti % face;
    const int p = f % n1 + 1, q = f / n1 + 1;
    (void)n2;
    int tgt, src;
    if (layer < nb1) {
        tgt = ng / 2 + 1 + layer;
        src = m - ng / 2 + layer;
    } else {
        tgt = m - (ng - 1) + (layer - nb1);
        src = 1 + (layer - nb1);
    }
    long long lt, ls;
    if (axis == 0) { lt = lin(g, tgt, p, q); ls = lin(g, src, p, q); }
    else if (axis == 1) { lt = lin(g, p, tgt, q); ls = lin(g, p, src, q); }
    else { lt = lin(g, p, q, tgt); ls = lin(g, p, q, src); }
    cx[lt] = cx[lt] + cx[ls];
    // Q5 (left-hand-side reading of fieldboundaries.F90:1938): the last
    // buffer row of the cury y-fold still holds curx(:,my,:)
    const float ysrc = (q5 && layer == nb1 - 1) ? cx[ls] : cy[ls];
    cy[lt] = cy[lt] + ysrc;
    cz[lt] = cz[lt] + cz[ls];
}

// cells written by one axis of the fold: both slabs of a face (slab < 0),
// or slab 0 (nghost/2 + 1 layers) or slab 1 (nghost/2 layers) alone
__host__ __device__ inline long long fold_cells(const Geom &g, int axis, int slab = -1) {
    const int ng = axis == 2 ? g.ngz : g.ng;
    const int n1 = axis == 0 ? g.my : g.mx, n2 = axis == 2 ? g.my : g.mz;
    const int layers = slab < 0 ? ng : slab == 0 ? ng / 2 + 1 : ng / 2;
    return (long long)n1 * n2 * layers;
}

// The two slabs' target layers (nghost/2+1 .. nghost and m-(nghost-1) ..
// m-(nghost/2+1)) are disjoint when the axis has at least nghost interior
// cells; below that they overlap and the slabs must be added in order.
// Each slab's sources never overlap a target layer of the same or the
// earlier slab while the axis has more than nghost/2 interior cells.
__host__ __device__ inline bool fold_in_one_pass(const Geom &g, int axis) {
    const int m = axis == 0 ? g.mx : axis == 1 ? g.my : g.mz;
    const int ng = axis == 2 ? g.ngz : g.ng;
    return m - ng >= ng;
}

// ---------------------------------------------------------------------------
// One pass of apply_filter1_opt (code/filter.F90:64-216), out-of-place:
// the one-layer ghost refresh is folded into the reads (R maps the
// refreshed layer to its periodic image), stencil cells get the 9/27-point
// sum in the reference's term order, all other cells the refreshed copy.
// The curz row range extends two rows (Q6, filter.F90:186,211).
// ---------------------------------------------------------------------------
struct RefreshMap {
    int m, ng, per;
    __device__ __forceinline__ int operator()(int t) const {
        if (!per) return t;
        if (t == ng / 2) return m - (ng / 2 + 1);
        if (t == m - ng / 2) return ng / 2 + 1;
        return t;
    }
};

// 27-point binomial sum of apply_filter1_opt in 3D (code/filter.F90:
// 130-160), in the reference's term order: the k plane's 9 terms, then
// the k-1 and k+1 planes' terms added one by one. a(di, dj, dk) is the
// (refreshed) input at offset (di, dj, dk) from the cell.
template <class Acc>
__device__ __forceinline__ float stencil27(const Acc &a) {
    const float w = 0.015625f;  // 1/64
    float s = 4.0f * w * a(-1, 0, 0) + 8.0f * w * a(0, 0, 0) + 4.0f * w * a(1, 0, 0) + 4.0f * w * a(0, -1, 0) +
              4.0f * w * a(0, 1, 0) + 2.0f * w * a(-1, 1, 0) + 2.0f * w * a(1, 1, 0) + 2.0f * w * a(-1, -1, 0) +
              2.0f * w * a(1, -1, 0);
    s = s + 2.0f * w * a(-1, 0, -1) + 4.0f * w * a(0, 0, -1) + 2.0f * w * a(1, 0, -1) + 2.0f * w * a(0, -1, -1) +
        2.0f * w * a(0, 1, -1) + 1.0f * w * a(-1, 1, -1) + 1.0f * w * a(1, 1, -1) + 1.0f * w * a(-1, -1, -1) +
        1.0f * w * a(1, -1, -1) + 2.0f * w * a(-1, 0, 1) + 4.0f * w * a(0, 0, 1) + 2.0f * w * a(1, 0, 1) +
        2.0f * w * a(0, -1, 1) + 2.0f * w * a(0, 1, 1) + 1.0f * w * a(-1, 1, 1) + 1.0f * w * a(1, 1, 1) +
        1.0f * w * a(-1, -1, 1) + 1.0f * w * a(1, -1, 1);
    return s;
}

template <int DIM>
__device__ __forceinline__ void filter_one(const Geom &g, const float *__restrict__ i0, const float *__restrict__ i1,
                                           const float *__restrict__ i2, float *o0, float *o1, float *o2,
                                           long long t) {
    const RefreshMap Rx{g.mx, g.ng, g.per[0]}, Ry{g.my, g.ng, g.per[1]}, Rz{g.mz, g.ngz, DIM == 3 ? g.per[2] : 0};
    const int ilo = g.ng / 2 + 1, ihi = g.mx - (g.ng / 2 + 1);
    const int jlo = g.ng / 2 + 1, jhi = g.my - (g.ng / 2 + 1);
    const int klo = DIM == 3 ? g.ngz / 2 + 1 : 1, khi = DIM == 3 ? g.mz - (g.ngz / 2 + 1) : 1;
    const int ti = (int)t;
    const int i = ti % g.mx + 1;
    const int r = ti / g.mx;
    const int j = r % g.my + 1;
    const int k = r / g.my + 1;
    const bool in_ik = i >= ilo && i <= ihi && k >= klo && k <= khi;
    const bool in_xy = in_ik && j >= jlo && j <= jhi;
    const bool in_z = in_ik && j >= jlo && j <= jhi + 2;
    const long long lr = lin(g, Rx(i), Ry(j), Rz(k));
    if (!in_z) {
        o0[t] = i0[lr];
        o1[t] = i1[lr];
        o2[t] = i2[lr];
        return;
    }
    const int im = Rx(i - 1), ip = Rx(i + 1), jm = Ry(j - 1), jp = Ry(j + 1);
    const int ii = Rx(i), jj = Ry(j);
#define TG_ST2(A, K)                                                                                  \
    (2.0f * 0.0625f * A[lin(g, im, jj, K)] + 4.0f * 0.0625f * A[lin(g, ii, jj, K)] +                 \
     2.0f * 0.0625f * A[lin(g, ip, jj, K)] + 2.0f * 0.0625f * A[lin(g, ii, jm, K)] +                 \
     2.0f * 0.0625f * A[lin(g, ii, jp, K)] + 1.0f * 0.0625f * A[lin(g, im, jp, K)] +                 \
     1.0f * 0.0625f * A[lin(g, ip, jp, K)] + 1.0f * 0.0625f * A[lin(g, im, jm, K)] +                 \
     1.0f * 0.0625f * A[lin(g, ip, jm, K)])
    float res[3];
#pragma unroll
    for (int comp = 0; comp < 3; comp++) {
        const float *A = comp == 0 ? i0 : comp == 1 ? i1 : i2;
        const bool st = comp == 2 ? in_z : in_xy;
        if (!st) {
            res[comp] = A[lr];
            continue;
        }
        if (DIM == 2) {
            res[comp] = TG_ST2(A, 1);
        } else {
            const int kk = Rz(k), km = Rz(k - 1), kp = Rz(k + 1);
            const int xs[3] = {im, ii, ip}, ys[3] = {jm, jj, jp}, zs[3] = {km, kk, kp};
            const float s = stencil27([&](int di, int dj, int dk) {
                return A[lin(g, xs[di + 1], ys[dj + 1], zs[dk + 1])];
            });
            res[comp] = s;
        }
    }
#undef TG_ST2
    o0[t] = res[0];
    o1[t] = res[1];
    o2[t] = res[2];
}

__device__ __forceinline__ void fixed_to_float_one(double inv, unsigned long long *f0, unsigned long long *f1,
                                                   unsigned long long *f2, float *c0, float *c1, float *c2,
                                                   long long t) {
    c0[t] = __double2float_rn(__ll2double_rn((long long)f0[t]) * inv);
    c1[t] = __double2float_rn(__ll2double_rn((long long)f1[t]) * inv);
    c2[t] = __double2float_rn(__ll2double_rn((long long)f2[t]) * inv);
    f0[t] = 0ull;
    f1[t] = 0ull;
    f2[t] = 0ull;
}

}  // namespace tg

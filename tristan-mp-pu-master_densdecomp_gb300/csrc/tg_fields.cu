// Field kernels of the GB300 TRISTAN-MP hot path (sm_103a).
//
// All arrays keep the reference's Fortran layout (mx,my,mz), x fastest, so a
// warp reads 32 consecutive x cells (coalesced 128-byte lines). Each kernel
// is one pass over its cells and is HBM-bound; the stencils round exactly as
// the reference (compiled without FMA contraction).
#include <cuda_runtime.h>

#include "tg_internal.cuh"

namespace tg {

static inline int blocks_for(long long n, int bs) {
    long long b = (n + bs - 1) / bs;
    if (b < 1) b = 1;
    if (b > 152 * 32) b = 152 * 32;
    return (int)b;
}

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

__global__ void k_ghost(Geom g, float *a, float *b, float *c, GhostAxis ax, GhostAxis ay, GhostAxis az,
                        long long nX, long long nY, long long nZ) {
    const long long total = nX + nY + nZ;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        int i, j, k;
        if (t < nX) {  // x-target layers, every j, k
            long long r = t;
            i = ax.target((int)(r % ax.nt));
            r /= ax.nt;
            j = (int)(r % g.my) + 1;
            k = (int)(r / g.my) + 1;
        } else if (t < nX + nY) {  // x non-target, y-target, every k
            long long r = t - nX;
            const int nnx = g.mx - ax.nt;
            i = ax.nontarget((int)(r % nnx));
            r /= nnx;
            j = ay.target((int)(r % ay.nt));
            k = (int)(r / ay.nt) + 1;
        } else {  // x, y non-target, z-target
            long long r = t - nX - nY;
            const int nnx = g.mx - ax.nt, nny = g.my - ay.nt;
            i = ax.nontarget((int)(r % nnx));
            r /= nnx;
            j = ay.nontarget((int)(r % nny));
            k = az.target((int)(r / nny));
        }
        const long long dst = lin(g, i, j, k);
        const long long src = lin(g, ax.image(i), ay.image(j), az.image(k));
        a[dst] = a[src];
        b[dst] = b[src];
        c[dst] = c[src];
    }
}

cudaError_t launch_ghost(const Geom &g, float *a, float *b, float *c, GhostKind kind, cudaStream_t st) {
    GhostAxis ax{g.mx, g.ng, g.per[0], ghost_targets(g.per[0], kind, g.ng, true), kind};
    GhostAxis ay{g.my, g.ng, g.per[1], ghost_targets(g.per[1], kind, g.ng, true), kind};
    GhostAxis az{g.mz, g.ngz, g.per[2], ghost_targets(g.per[2], kind, g.ngz, g.dims == 3), kind};
    const long long nX = (long long)ax.nt * g.my * g.mz;
    const long long nY = (long long)(g.mx - ax.nt) * ay.nt * g.mz;
    const long long nZ = (long long)(g.mx - ax.nt) * (g.my - ay.nt) * az.nt;
    const long long total = nX + nY + nZ;
    if (total == 0) return cudaSuccess;
    k_ghost<<<blocks_for(total, 256), 256, 0, st>>>(g, a, b, c, ax, ay, az, nX, nY, nZ);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Update ranges of advance_b_halfstep / advance_e_fullstep for one rank
// (code/fields.F90:593-665, :746-821).
// ---------------------------------------------------------------------------
static void b_range(const Geom &g, int axis, int &a1, int &a2) {
    const int m = axis == 0 ? g.mx : axis == 1 ? g.my : g.mz;
    const int ng = axis == 2 ? g.ngz : g.ng;
    if (axis == 2 && g.dims == 2) { a1 = 1; a2 = 1; return; }
    if (g.per[axis]) { a1 = ng / 2 + 1; a2 = m - (ng / 2 + 1); }
    else { a1 = 1; a2 = m - 1; }
}

static void e_range(const Geom &g, int axis, int &a1, int &a2) {
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
__global__ void k_advance_b(Geom g, Box bx_, float cst, const float *__restrict__ ex, const float *__restrict__ ey,
                            const float *__restrict__ ez, float *bx, float *by, float *bz) {
    const long long total = (long long)bx_.ni * bx_.nj * bx_.nk;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % bx_.ni) + bx_.i1;
        const long long r = t / bx_.ni;
        const int j = (int)(r % bx_.nj) + bx_.j1;
        const int k = (int)(r / bx_.nj) + bx_.k1;
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
}

template <int DIM>
__global__ void k_advance_e(Geom g, Box b_, float cst, float *ex, float *ey, float *ez, const float *__restrict__ bx,
                            const float *__restrict__ by, const float *__restrict__ bz) {
    const long long total = (long long)b_.ni * b_.nj * b_.nk;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % b_.ni) + b_.i1;
        const long long r = t / b_.ni;
        const int j = (int)(r % b_.nj) + b_.j1;
        const int k = (int)(r / b_.nj) + b_.k1;
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
// per axis, cur(ng/2+1..ng) += cur(m-ng/2..m) and
// cur(m-(ng-1)..m-(ng/2+1)) += cur(1..ng/2). Targets and sources are
// disjoint, so one thread per target cell. Axis order x, y, z.
// ---------------------------------------------------------------------------
__global__ void k_fold(Geom g, int axis, int m, int ng, float *cx, float *cy, float *cz, int q5) {
    const int nb1 = ng / 2 + 1, nb2 = ng / 2;
    const int n1 = axis == 0 ? g.my : g.mx;                 // first face extent
    const int n2 = axis == 2 ? g.my : g.mz;                 // second face extent
    const long long face = (long long)n1 * n2;
    const long long total = face * (nb1 + nb2);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int layer = (int)(t / face);
        const long long f = t % face;
        const int p = (int)(f % n1) + 1, q = (int)(f / n1) + 1;
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
}

cudaError_t launch_fold(const Geom &g, const Params &P, float *const *cur, cudaStream_t st) {
    for (int axis = 0; axis < 3; axis++) {
        if (axis == 2 && g.dims == 2) break;
        if (!g.per[axis]) continue;
        const int m = axis == 0 ? g.mx : axis == 1 ? g.my : g.mz;
        const int ng = axis == 2 ? g.ngz : g.ng;
        const int n1 = axis == 0 ? g.my : g.mx, n2 = axis == 2 ? g.my : g.mz;
        const long long total = (long long)n1 * n2 * ng;
        const int q5 = (axis == 1) && (P.quirks & TG_QUIRK_Q5_LHS);
        k_fold<<<blocks_for(total, 256), 256, 0, st>>>(g, axis, m, ng, cur[0], cur[1], cur[2], q5);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
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

template <int DIM>
__global__ void __launch_bounds__(256) k_filter(Geom g, const float *__restrict__ i0, const float *__restrict__ i1,
                                                const float *__restrict__ i2, float *o0, float *o1, float *o2) {
    const RefreshMap Rx{g.mx, g.ng, g.per[0]}, Ry{g.my, g.ng, g.per[1]}, Rz{g.mz, g.ngz, DIM == 3 ? g.per[2] : 0};
    const int ilo = g.ng / 2 + 1, ihi = g.mx - (g.ng / 2 + 1);
    const int jlo = g.ng / 2 + 1, jhi = g.my - (g.ng / 2 + 1);
    const int klo = DIM == 3 ? g.ngz / 2 + 1 : 1, khi = DIM == 3 ? g.mz - (g.ngz / 2 + 1) : 1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.lot;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.mx) + 1;
        const long long r = t / g.mx;
        const int j = (int)(r % g.my) + 1;
        const int k = (int)(r / g.my) + 1;
        const bool in_ik = i >= ilo && i <= ihi && k >= klo && k <= khi;
        const bool in_xy = in_ik && j >= jlo && j <= jhi;
        const bool in_z = in_ik && j >= jlo && j <= jhi + 2;
        const long long lr = lin(g, Rx(i), Ry(j), Rz(k));
        if (!in_z) {
            o0[t] = i0[lr];
            o1[t] = i1[lr];
            o2[t] = i2[lr];
            continue;
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
                const float w = 0.015625f;  // 1/64
                const int kk = Rz(k), km = Rz(k - 1), kp = Rz(k + 1);
                float s = 4.0f * w * A[lin(g, im, jj, kk)] + 8.0f * w * A[lin(g, ii, jj, kk)] +
                          4.0f * w * A[lin(g, ip, jj, kk)] + 4.0f * w * A[lin(g, ii, jm, kk)] +
                          4.0f * w * A[lin(g, ii, jp, kk)] + 2.0f * w * A[lin(g, im, jp, kk)] +
                          2.0f * w * A[lin(g, ip, jp, kk)] + 2.0f * w * A[lin(g, im, jm, kk)] +
                          2.0f * w * A[lin(g, ip, jm, kk)];
                s = s + 2.0f * w * A[lin(g, im, jj, km)] + 4.0f * w * A[lin(g, ii, jj, km)] +
                    2.0f * w * A[lin(g, ip, jj, km)] + 2.0f * w * A[lin(g, ii, jm, km)] +
                    2.0f * w * A[lin(g, ii, jp, km)] + 1.0f * w * A[lin(g, im, jp, km)] +
                    1.0f * w * A[lin(g, ip, jp, km)] + 1.0f * w * A[lin(g, im, jm, km)] +
                    1.0f * w * A[lin(g, ip, jm, km)] + 2.0f * w * A[lin(g, im, jj, kp)] +
                    4.0f * w * A[lin(g, ii, jj, kp)] + 2.0f * w * A[lin(g, ip, jj, kp)] +
                    2.0f * w * A[lin(g, ii, jm, kp)] + 2.0f * w * A[lin(g, ii, jp, kp)] +
                    1.0f * w * A[lin(g, im, jp, kp)] + 1.0f * w * A[lin(g, ip, jp, kp)] +
                    1.0f * w * A[lin(g, im, jm, kp)] + 1.0f * w * A[lin(g, ip, jm, kp)];
                res[comp] = s;
            }
        }
#undef TG_ST2
        o0[t] = res[0];
        o1[t] = res[1];
        o2[t] = res[2];
    }
}

cudaError_t launch_filter_pass(const Geom &g, float *const *in, float *const *out, cudaStream_t st) {
    if (g.dims == 3)
        k_filter<3><<<blocks_for(g.lot, 256), 256, 0, st>>>(g, in[0], in[1], in[2], out[0], out[1], out[2]);
    else
        k_filter<2><<<blocks_for(g.lot, 256), 256, 0, st>>>(g, in[0], in[1], in[2], out[0], out[1], out[2]);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Primal-averaged copies for the 3D gather (code/particles_movedeposit.F90:
// 395-404): cshift(.,-1) wraps over the whole local array.
// ---------------------------------------------------------------------------
__global__ void k_primal(Geom g, const float *__restrict__ ex, const float *__restrict__ ey,
                         const float *__restrict__ ez, const float *__restrict__ bx, const float *__restrict__ by,
                         const float *__restrict__ bz, float *pex, float *pey, float *pez, float *pbx, float *pby,
                         float *pbz) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.lot;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.mx) + 1;
        const long long r = t / g.mx;
        const int j = (int)(r % g.my) + 1;
        const int k = (int)(r / g.my) + 1;
        const int im = i == 1 ? g.mx : i - 1, jm = j == 1 ? g.my : j - 1, km = k == 1 ? g.mz : k - 1;
        const long long lxm = lin(g, im, j, k), lym = lin(g, i, jm, k), lzm = lin(g, i, j, km);
        pex[t] = 0.5f * (ex[t] + ex[lxm]);
        pey[t] = 0.5f * (ey[t] + ey[lym]);
        pez[t] = 0.5f * (ez[t] + ez[lzm]);
        pbx[t] = 0.5f * (bx[t] + bx[lym]);
        pby[t] = 0.5f * (by[t] + by[lxm]);
        pbz[t] = 0.5f * (0.5f * (bz[t] + bz[lxm]) + 0.5f * (bz[lym] + bz[lin(g, im, jm, k)]));
    }
}

cudaError_t launch_primal(const Geom &g, float *const *f, float *const *pf, cudaStream_t st) {
    k_primal<<<blocks_for(g.lot, 256), 256, 0, st>>>(g, f[0], f[1], f[2], f[3], f[4], f[5], pf[0], pf[1], pf[2],
                                                     pf[3], pf[4], pf[5]);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// int64 fixed-point accumulators -> float currents; clears the accumulators
// ---------------------------------------------------------------------------
__global__ void k_fixed_to_float(long long n, double inv, unsigned long long *f0, unsigned long long *f1,
                                 unsigned long long *f2, float *c0, float *c1, float *c2) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        c0[t] = __double2float_rn(__ll2double_rn((long long)f0[t]) * inv);
        c1[t] = __double2float_rn(__ll2double_rn((long long)f1[t]) * inv);
        c2[t] = __double2float_rn(__ll2double_rn((long long)f2[t]) * inv);
        f0[t] = 0ull;
        f1[t] = 0ull;
        f2[t] = 0ull;
    }
}

cudaError_t launch_fixed_to_float(const Geom &g, const Params &P, unsigned long long *const *fx, float *const *cur,
                                  cudaStream_t st) {
    k_fixed_to_float<<<blocks_for(g.lot, 256), 256, 0, st>>>(g.lot, P.fx_inv, fx[0], fx[1], fx[2], cur[0], cur[1],
                                                             cur[2]);
    return cudaGetLastError();
}

}  // namespace tg

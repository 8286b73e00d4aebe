// FP64 diagnostics of the GB300 TRISTAN-MP hot path (sm_103a).
//
// Gauss's law with the binomial filter: the deposit is charge conserving
// and the filter (a periodic convolution) commutes with the divergence, so
// with a neutral start div E = F^ntimes(rho) at every lap, rho the charge
// deposited with the same B-spline. Per lap:
//  k_diag_particles  one CTA per tile: rho in an int64 fixed-point shared
//                    window (products in FP32, one rounding to 2^-fx_shift,
//                    so the sum is order independent), kinetic energy
//                    (gamma-1 = u^2/(gamma+1) in FP32) and momentum summed
//                    in FP64;
//  k_rho_to_int      fixed point -> the filter's finer integer grid;
//  k_filter_rho_pass one binomial pass on the periodic interior, as
//                    [1, 2, 1] / 4 along each axis in turn in int64 (each
//                    step rounded to the grid), all axes of a pass in one
//                    kernel through a shared-memory tile;
//  k_diag_fields     FP64 reductions of |div E - F(rho)|^2, |F(rho)|^2 and
//                    the total charge (div E - F(rho) is a small difference),
//                    compensated FP32 sums of the field energies and E x B
//                    momentum;
//  k_diag_finish     writes the lap's record into the history ring.
// GB300 has little FP64 throughput, so FP64 is used only where the sums
// need it (accumulators and the Gauss residual).
#include <cuda_runtime.h>

#include "tg_particles.cuh"
#include "tg_spectrum.cuh"

namespace tg {


struct DiagArgs {
    Geom g;
    Params P;
    Species sp[2];
    const int *tstart[2];
    unsigned long long *rhofx;  // interior, periodic
    double *acc;                // [D_N]
    float mass[2];              // |q/qm| per species
    int *status;
    int only;                   // 0 both species, 1 ions only, 2 electrons only
};

// resident CTAs per SM the particle pass's registers are sized for, per
// dimension
#ifndef TG_DIAG_MINB_2D
#define TG_DIAG_MINB_2D 4
#endif
#ifndef TG_DIAG_MINB_3D
#define TG_DIAG_MINB_3D 4
#endif
template <int DIM, int ORDER>
__global__ void __launch_bounds__(256, DIM == 3 ? TG_DIAG_MINB_3D : TG_DIAG_MINB_2D) k_diag_particles(DiagArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    unsigned *winlo = reinterpret_cast<unsigned *>(smem_raw);
    int *winhi = reinterpret_cast<int *>(smem_raw) + a.g.wcells;
    const Geom &g = a.g;
    const int tile = blockIdx.x;
    const int tix = tile % g.ntx, tiy = (tile / g.ntx) % g.nty, tiz = tile / (g.ntx * g.nty);
    const int wx0 = g.ox + tix * g.tx - g.wlo, wy0 = g.oy + tiy * g.ty - g.wlo;
    const int wz0 = DIM == 3 ? g.oz + tiz * g.tz - g.wlo : 1;
    for (int t = threadIdx.x; t < 2 * g.wcells; t += blockDim.x) winlo[t] = 0u;
    __syncthreads();
    double part[5] = {0, 0, 0, 0, 0};  // eki, eke, px, py, pz
    // the window is exact for up to 65536 contributions per node: a denser
    // tile deposits straight to global memory
    const int s0 = a.only == 2 ? 1 : 0, s1 = a.only == 1 ? 1 : 2;
    int nt = 0;
    for (int s = s0; s < s1; s++) nt += a.tstart[s][tile + 1] - a.tstart[s][tile];
    const bool use_win = nt <= TG_WIN_BATCH;
    for (int s = s0; s < s1; s++) {
        const Species sp = a.sp[s];
        const int beg = a.tstart[s][tile], end = a.tstart[s][tile + 1];
        const float qs = a.P.qs[s], m = a.mass[s];
        // per-thread compensated FP32 sums, one FP64 add per thread and species
        // (GB300 issues FP64 at a small fraction of the FP32 rate)
        float ks[4] = {0, 0, 0, 0}, kc[4] = {0, 0, 0, 0};
        // the next particle's record is loaded before this one is deposited,
        // so its memory latency overlaps the deposit
        int n = beg + threadIdx.x;
        int cell = n < end ? sp.cell[n] : -1;
        float ox = 0.f, oy = 0.f, oz = 0.f, ch = 0.f, u = 0.f, v = 0.f, w = 0.f;
        if (n < end) {
            ox = sp.ox[n]; oy = sp.oy[n]; oz = DIM == 3 ? sp.oz[n] : 0.0f;
            ch = sp.ch[n]; u = sp.u[n]; v = sp.v[n]; w = sp.w[n];
        }
        while (n < end) {
            const int ccell = cell;
            const float cox = ox, coy = oy, coz = oz, cch = ch, cu = u, cv = v, cw = w;
            n += blockDim.x;
            if (n < end) {
                cell = sp.cell[n];
                ox = sp.ox[n]; oy = sp.oy[n]; oz = DIM == 3 ? sp.oz[n] : 0.0f;
                ch = sp.ch[n]; u = sp.u[n]; v = sp.v[n]; w = sp.w[n];
            }
            if (ccell < 0) continue;
            int i, j, k;
            cell_ijk(g, ccell, i, j, k);
            const float q = cch * qs;
            rho_deposit<DIM, ORDER>(g, a.P.fx_scale, i, j, k, cox, coy, coz, q, winlo, winhi, wx0, wy0, wz0,
                                    use_win, a.rhofx);
            const float u2 = cu * cu + cv * cv + cw * cw;
            const float gm1 = u2 / (sqrtf(1.0f + u2) + 1.0f);
            const float mc = m * cch;
            const float terms[4] = {gm1 * mc, mc * cu, mc * cv, mc * cw};
#pragma unroll
            for (int t4 = 0; t4 < 4; t4++) {  // Kahan summation
                const float y = terms[t4] - kc[t4];
                const float t = ks[t4] + y;
                kc[t4] = (t - ks[t4]) - y;
                ks[t4] = t;
            }
        }
        part[s] += (double)ks[0] - (double)kc[0];
        part[2] += (double)ks[1] - (double)kc[1];
        part[3] += (double)ks[2] - (double)kc[2];
        part[4] += (double)ks[3] - (double)kc[3];
    }
    __syncthreads();
    rho_flush<DIM>(g, winlo, winhi, wx0, wy0, wz0, a.rhofx);
    block_accumulate<5>(part, a.acc, D_EKI);
}

// fixed point -> the filter's integer grid: 16 more fraction bits, so the
// rounding of the filter's divisions stays far below the Gauss residual; a
// sum of 2^47 units or more (2^17 full particle charges on one node) would
// overflow the filter and is flagged. The accumulator is cleared for the
// next lap.
#define TG_RHO_SHIFT 16
__global__ void k_rho_to_int(long long n, unsigned long long *fx, long long *rho, int *status) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const long long v = (long long)fx[t];
        if (v >= (1LL << 47) || v <= -(1LL << 47)) atomicOr(status, ST_CHARGE_GRID);
        rho[t] = (long long)((unsigned long long)v << TG_RHO_SHIFT);
        fx[t] = 0ull;
    }
}

static int rgrid(int rows) { return rows < 152 * 16 ? (rows < 1 ? 1 : rows) : 152 * 16; }

// One binomial pass on the periodic interior (nx, ny, nz) is the product of
// [1, 2, 1] / 4 along each axis (the current filter's 9 / 27-point weights),
// applied here to the charge on its integer grid: each axis step is
// (l + 2 c + r + 2) >> 2 in int64, rounded to the grid (2^-(fx_shift + 16)
// of the fixed-point unit), integer work where FP64 would set the pace on
// this GPU. A CTA loads its tile with a one-cell halo (periodic images) into
// shared memory and steps along x over the halo rows too, then along y, then
// z, so the array crosses HBM once per pass.
#define TG_F64_TX 32
#define TG_F64_TY(DIM) ((DIM) == 3 ? 8 : 16)
#define TG_F64_TZ(DIM) ((DIM) == 3 ? 8 : 1)
static size_t filter64_smem(int dims) {
    const int hx = TG_F64_TX + 2, hy = TG_F64_TY(dims) + 2, hz = dims == 3 ? TG_F64_TZ(dims) + 2 : 1;
    return (size_t)(hz * hy * hx + hz * hy * TG_F64_TX) * sizeof(long long);
}

__device__ __forceinline__ int wrap_n(int i, int n) {
    i %= n;
    return i < 0 ? i + n : i;
}

__device__ __forceinline__ long long binom_step(long long l, long long c, long long r) {
    return (l + 2 * c + r + 2) >> 2;
}

template <int DIM>
__global__ void __launch_bounds__(256) k_filter_rho_pass(int nx, int ny, int nz, const long long *__restrict__ in,
                                                         long long *__restrict__ out) {
    constexpr int TX = TG_F64_TX, TY = TG_F64_TY(DIM), TZ = TG_F64_TZ(DIM);
    constexpr int HX = TX + 2, HY = TY + 2, HZ = DIM == 3 ? TZ + 2 : 1;
    extern __shared__ __align__(16) long long rhos[];
    long long *s_in = rhos;                // [HZ][HY][HX]; later the y step [HZ][TY][TX]
    long long *s_x = rhos + HZ * HY * HX;  // [HZ][HY][TX]
    const int a0 = blockIdx.x * TX, b0 = blockIdx.y * TY, c0 = blockIdx.z * TZ;
    for (int t = threadIdx.x; t < HZ * HY * HX; t += blockDim.x) {
        const int lx = t % HX, r = t / HX, ly = r % HY, lz = r / HY;
        const int a = wrap_n(a0 - 1 + lx, nx), b = wrap_n(b0 - 1 + ly, ny);
        const int c = DIM == 3 ? wrap_n(c0 - 1 + lz, nz) : 0;
        s_in[t] = in[((long long)c * ny + b) * nx + a];
    }
    __syncthreads();
    for (int t = threadIdx.x; t < HZ * HY * TX; t += blockDim.x) {
        const int lx = t % TX, row = t / TX;
        const long long *p = s_in + row * HX + lx;
        s_x[t] = binom_step(p[0], p[1], p[2]);
    }
    __syncthreads();
    long long *s_y = s_in;  // [HZ][TY][TX]
    for (int t = threadIdx.x; t < HZ * TY * TX; t += blockDim.x) {
        const int lx = t % TX, r = t / TX, ly = r % TY, lz = r / TY;
        const long long *p = s_x + (lz * HY + ly) * TX + lx;
        s_y[t] = binom_step(p[0], p[TX], p[2 * TX]);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < TZ * TY * TX; t += blockDim.x) {
        const int lx = t % TX, r = t / TX, ly = r % TY, lz = r / TY;
        const int a = a0 + lx, b = b0 + ly, c = c0 + lz;
        if (a >= nx || b >= ny || c >= nz) continue;
        long long v;
        if (DIM == 3) {
            const long long *p = s_y + (lz * TY + ly) * TX + lx;
            v = binom_step(p[0], p[TY * TX], p[2 * TY * TX]);
        } else {
            v = s_y[ly * TX + lx];
        }
        out[((long long)c * ny + b) * nx + a] = v;
    }
}

template <int DIM>
__global__ void __launch_bounds__(256) k_diag_fields(Geom g, const float *__restrict__ ex, const float *__restrict__ ey,
                                                     const float *__restrict__ ez, const float *__restrict__ bx,
                                                     const float *__restrict__ by, const float *__restrict__ bz,
                                                     const long long *__restrict__ rho, double inv, double *acc) {
    const int nx = g.mx - g.ng, ny = g.my - g.ng, nz = DIM == 3 ? g.mz - g.ngz : 1;
    const int lo = g.ng / 2 + 1, loz = DIM == 3 ? g.ngz / 2 + 1 : 1;
    double v[3] = {0, 0, 0};  // res2 rho2 charge: FP64 (the residual is a small difference)
    // field energies and momentum eE eB fx fy fz: per-thread compensated FP32
    // sums, one FP64 conversion per thread (GB300 issues FP64 at a small
    // fraction of the FP32 rate)
    float ks[5] = {0, 0, 0, 0, 0}, kc[5] = {0, 0, 0, 0, 0};
    // rows (one y, z) over the blocks, cells of a row over the threads
    for (int row = blockIdx.x; row < ny * nz; row += gridDim.x)
    for (int a = threadIdx.x; a < nx; a += blockDim.x) {
        const long long t = (long long)row * nx + a;
        const int b = row % ny, c = row / ny;
        const int i = lo + a, j = lo + b, k = loz + c;
        const long long l = lin(g, i, j, k);
        const int im = a == 0 ? lo + nx - 1 : i - 1, jm = b == 0 ? lo + ny - 1 : j - 1;
        double div = (double)ex[l] - (double)ex[lin(g, im, j, k)] + (double)ey[l] - (double)ey[lin(g, i, jm, k)];
        if (DIM == 3) {
            const int km = c == 0 ? loz + nz - 1 : k - 1;
            div += (double)ez[l] - (double)ez[lin(g, i, j, km)];
        }
        const double rh = __ll2double_rn(rho[t]) * inv;
        const double res = div - rh;
        v[0] += res * res;
        v[1] += rh * rh;
        v[2] += rh;
        const float e0 = ex[l], e1 = ey[l], e2 = ez[l], b0 = bx[l], b1 = by[l], b2 = bz[l];
        const float terms[5] = {0.5f * (e0 * e0 + e1 * e1 + e2 * e2), 0.5f * (b0 * b0 + b1 * b1 + b2 * b2),
                                e1 * b2 - e2 * b1, e2 * b0 - e0 * b2, e0 * b1 - e1 * b0};
#pragma unroll
        for (int q = 0; q < 5; q++) {  // Kahan summation
            const float y = terms[q] - kc[q];
            const float t2 = ks[q] + y;
            kc[q] = (t2 - ks[q]) - y;
            ks[q] = t2;
        }
    }
    double first[5] = {v[0], v[1], v[2], (double)ks[0] - (double)kc[0], (double)ks[1] - (double)kc[1]};
    block_accumulate<5>(first, acc, D_RES2);
    __syncthreads();
    double second[3] = {(double)ks[2] - (double)kc[2], (double)ks[3] - (double)kc[3], (double)ks[4] - (double)kc[4]};
    block_accumulate<3>(second, acc, D_FX);
}

// copy the lap's accumulators into the history ring and clear them
__global__ void k_diag_finish(double *acc, double *hist, int cap, unsigned long long *counter) {
    const unsigned long long slot = *counter % (unsigned long long)cap;
    if (threadIdx.x < D_N) {
        hist[slot * D_N + threadIdx.x] = acc[threadIdx.x];
        acc[threadIdx.x] = 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) *counter += 1ull;
}

// ---------------------------------------------------------------------------
// grid moments (meanq_fld_cur, code/output.F90:5222-5482): every particle
// adds its quantity and its weight to the cells of a box around its cell
// (FP64 atomics, rounded to single once); then the ghost fold, the division
// by the box size and, for velocity-like moments, by the weight
// ---------------------------------------------------------------------------
__device__ __forceinline__ void moment_box(const Geom &g, int idx, int idy, int idz, int i, int j, int k, int &lx1,
                                           int &lx2, int &ly1, int &ly2, int &lz1, int &lz2) {
    lz1 = max(k - idz, 1);
    lz2 = min(k + idz, g.mz);
    if (g.dims == 2) {
        lz1 = 1;
        lz2 = 1;
    }
    ly1 = max(j - idy, 1);
    ly2 = min(j + idy, g.my);
    lx1 = max(i - idx, 1);
    lx2 = min(i + idx, g.mx);
}

template <int DIM>
__global__ void __launch_bounds__(256) k_moments(Geom g, Species si, Species se, const long long *count, int kind,
                                                 int idx, int idy, int idz, double *num, double *den) {
    const long long n0 = count[0], n1 = count[1];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n0 + n1;
         t += (long long)gridDim.x * blockDim.x) {
        const bool ion = t < n0;
        const Species &sp = ion ? si : se;
        const long long n = ion ? t : t - n0;
        if (sp.cell[n] < 0) continue;
        float x, y, z;
        load_pos<DIM>(g, sp, n, x, y, z);
        const float u = sp.u[n], v = sp.v[n], w = sp.w[n], ch = sp.ch[n];
        const float gamprt = 1.0f / sqrtf(1.0f + u * u + v * v + w * w);
        float ax = 0.0f, ay = 0.0f;
        switch (kind) {
        case 0: ax = ch; break;
        case 1: if (ion) ax = ch; break;
        case 2: ax = u * gamprt * ch; ay = ch; break;
        case 3: ax = v * gamprt * ch; ay = ch; break;
        case 4: ax = w * gamprt * ch; ay = ch; break;
        case 5: if (ion) { ax = u * gamprt * ch; ay = ch; } break;
        case 6: if (ion) { ax = v * gamprt * ch; ay = ch; } break;
        case 7: if (ion) { ax = w * gamprt * ch; ay = ch; } break;
        case 8: ax = u * ch; ay = ch; break;
        case 9: ax = v * ch; ay = ch; break;
        case 10: ax = w * ch; ay = ch; break;
        case 11: if (ion) { ax = u * ch; ay = ch; } break;
        case 12: if (ion) { ax = v * ch; ay = ch; } break;
        case 13: if (ion) { ax = w * ch; ay = ch; } break;
        case 14: if (!ion) { ax = (1.0f / gamprt - 1.0f) * ch; ay = ch; } break;
        case 15: if (ion) { ax = (1.0f / gamprt - 1.0f) * ch; ay = ch; } break;
        default: break;
        }
        if (ax == 0.0f && ay == 0.0f) continue;
        int lx1, lx2, ly1, ly2, lz1, lz2;
        moment_box(g, idx, idy, idz, (int)x, (int)y, DIM == 3 ? (int)z : 1, lx1, lx2, ly1, ly2, lz1, lz2);
        for (int kk = lz1; kk <= lz2; kk++)
            for (int jj = ly1; jj <= ly2; jj++)
                for (int ii = lx1; ii <= lx2; ii++) {
                    const long long l = lin(g, ii, jj, kk);
                    if (ax != 0.0f) atomicAdd(num + l, (double)ax);
                    if (ay != 0.0f) atomicAdd(den + l, (double)ay);
                }
    }
}

__global__ void k_moments_round(long long lot, double *num, double *den, float *fn, float *fd, float *fz) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < lot;
         t += (long long)gridDim.x * blockDim.x) {
        fn[t] = __double2float_rn(num[t]);
        fd[t] = __double2float_rn(den[t]);
        fz[t] = 0.0f;
        num[t] = 0.0;
        den[t] = 0.0;
    }
}

__global__ void k_moments_box(Geom g, int kind, int idx, int idy, int idz, float *fn, float *fd) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < g.lot;
         t += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(t % g.mx) + 1;
        const long long r = t / g.mx;
        const int j = (int)(r % g.my) + 1;
        const int k = (int)(r / g.my) + 1;
        int lx1, lx2, ly1, ly2, lz1, lz2;
        moment_box(g, idx, idy, idz, i, j, k, lx1, lx2, ly1, ly2, lz1, lz2);
        const float box = (float)((lx2 - lx1 + 1) * (ly2 - ly1 + 1) * (lz2 - lz1 + 1));
        float a = fn[t] / box;
        const float b = fd[t] / box;
        if (kind >= 2) a = b != 0.0f ? a / b : 0.0f;
        fn[t] = a;
        fd[t] = b;
    }
}

static int dgrid(long long n);

cudaError_t launch_moments(const Geom &g, const Params &P, const Species *sp, const long long *count, long long hint,
                           int kind, int idx, int idy, int idz, double *num, double *den, float *const *f3,
                           cudaStream_t st) {
    const int grid = dgrid(hint);
    if (g.dims == 3) k_moments<3><<<grid, 256, 0, st>>>(g, sp[0], sp[1], count, kind, idx, idy, idz, num, den);
    else k_moments<2><<<grid, 256, 0, st>>>(g, sp[0], sp[1], count, kind, idx, idy, idz, num, den);
    k_moments_round<<<dgrid(g.lot), 256, 0, st>>>(g.lot, num, den, f3[0], f3[1], f3[2]);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if ((e = launch_fold(g, P, f3, st)) != cudaSuccess) return e;
    k_moments_box<<<dgrid(g.lot), 256, 0, st>>>(g, kind, idx, idy, idz, f3[0], f3[1]);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// output_tot (code/output.F90:2494-3884): one variable of the .tot. field
// file sampled every istep nodes. E and B go through interpolfld
// (code/output.F90:4995-5127): each staggered component averaged to the node
// and tri-linearly interpolated at (x, y, z), in the reference's order of
// operations; the output nodes are integer positions, so the interpolation
// weights are zero, but the expressions are kept whole so that the roundings
// (signed zeros included) are the reference's.
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ float interpolfld_one(const Geom &g, int comp, const float *__restrict__ a, float x,
                                                 float y, float z) {
    int i = (int)x, j = (int)y, k = DIM == 3 ? (int)z : 1;
    const float dx = x - (float)i, dy = y - (float)j;
    float dz = DIM == 3 ? z - (float)k : 0.0f;
    if (i == 1) i = 2;
    if (i == g.mx) i = g.mx - 1;
    if (j == 1) j = 2;
    if (j == g.my) j = g.my - 1;
    if (DIM == 3) {
        if (k == 1) k = 2;
        if (k == g.mz) k = g.mz - 1;
    }
    const long long ix = 1, iy = g.sy, iz = DIM == 3 ? g.sz : 0;
    // Fortran's 1-based l = i + iy (j - 1) + iz (k - 1) as a 0-based pointer
    const float *A = a + (i - 1) + iy * (j - 1) + iz * (k - 1);
    auto f_ = [&](long long o) { return A[o]; };
    float f, h;
    switch (comp) {
    case 0:  // ex: half-integer in x
        f = f_(0) + f_(-ix) + dx * (f_(ix) - f_(-ix));
        f = f + dy * (f_(iy) + f_(-ix + iy) + dx * (f_(ix + iy) - f_(-ix + iy)) - f);
        h = f_(iz) + f_(-ix + iz) + dx * (f_(ix + iz) - f_(-ix + iz));
        h = h + dy * (f_(iy + iz) + f_(-ix + iy + iz) + dx * (f_(ix + iy + iz) - f_(-ix + iy + iz)) - h);
        return (f + dz * (h - f)) * 0.5f;
    case 1:  // ey
        f = f_(0) + f_(-iy) + dy * (f_(iy) - f_(-iy));
        f = f + dz * (f_(iz) + f_(-iy + iz) + dy * (f_(iy + iz) - f_(-iy + iz)) - f);
        h = f_(ix) + f_(-iy + ix) + dy * (f_(iy + ix) - f_(-iy + ix));
        h = h + dz * (f_(iz + ix) + f_(-iy + iz + ix) + dy * (f_(iy + iz + ix) - f_(-iy + iz + ix)) - h);
        return (f + dx * (h - f)) * 0.5f;
    case 2:  // ez
        f = f_(0) + f_(-iz) + dz * (f_(iz) - f_(-iz));
        f = f + dx * (f_(ix) + f_(-iz + ix) + dz * (f_(iz + ix) - f_(-iz + ix)) - f);
        h = f_(iy) + f_(-iz + iy) + dz * (f_(iz + iy) - f_(-iz + iy));
        h = h + dx * (f_(ix + iy) + f_(-iz + ix + iy) + dz * (f_(iz + ix + iy) - f_(-iz + ix + iy)) - h);
        return (f + dy * (h - f)) * 0.5f;
    case 3:  // bx: half-integer in y and z
        f = f_(-iy) + f_(-iy - iz) + dz * (f_(-iy + iz) - f_(-iy - iz));
        f = f_(0) + f_(-iz) + dz * (f_(iz) - f_(-iz)) + f +
            dy * (f_(iy) + f_(iy - iz) + dz * (f_(iy + iz) - f_(iy - iz)) - f);
        h = f_(ix - iy) + f_(ix - iy - iz) + dz * (f_(ix - iy + iz) - f_(ix - iy - iz));
        h = f_(ix) + f_(ix - iz) + dz * (f_(ix + iz) - f_(ix - iz)) + h +
            dy * (f_(ix + iy) + f_(ix + iy - iz) + dz * (f_(ix + iy + iz) - f_(ix + iy - iz)) - h);
        return (f + dx * (h - f)) * 0.25f;
    case 4:  // by
        f = f_(-iz) + f_(-iz - ix) + dx * (f_(-iz + ix) - f_(-iz - ix));
        f = f_(0) + f_(-ix) + dx * (f_(ix) - f_(-ix)) + f +
            dz * (f_(iz) + f_(iz - ix) + dx * (f_(iz + ix) - f_(iz - ix)) - f);
        h = f_(iy - iz) + f_(iy - iz - ix) + dx * (f_(iy - iz + ix) - f_(iy - iz - ix));
        h = f_(iy) + f_(iy - ix) + dx * (f_(iy + ix) - f_(iy - ix)) + h +
            dz * (f_(iy + iz) + f_(iy + iz - ix) + dx * (f_(iy + iz + ix) - f_(iy + iz - ix)) - h);
        return (f + dy * (h - f)) * 0.25f;
    default:  // bz
        f = f_(-ix) + f_(-ix - iy) + dy * (f_(-ix + iy) - f_(-ix - iy));
        f = f_(0) + f_(-iy) + dy * (f_(iy) - f_(-iy)) + f +
            dx * (f_(ix) + f_(ix - iy) + dy * (f_(ix + iy) - f_(ix - iy)) - f);
        h = f_(iz - ix) + f_(iz - ix - iy) + dy * (f_(iz - ix + iy) - f_(iz - ix - iy));
        h = f_(iz) + f_(iz - iy) + dy * (f_(iz + iy) - f_(iz - iy)) + h +
            dx * (f_(iz + ix) + f_(iz + ix - iy) + dy * (f_(iz + ix + iy) - f_(iz + ix - iy)) - h);
        return (f + dz * (h - f)) * 0.25f;
    }
}

// out[a + n0 (b + n1 c)] = variable at node (start + istep (a, b, c)):
// comp 0-5 interpolated E / B plus the constant external field add, comp < 0
// the array's value at the node
template <int DIM>
__global__ void __launch_bounds__(256) k_output_sample(Geom g, int comp, const float *__restrict__ a, float add,
                                                       int3 start, int3 n, int istep, float *out) {
    const long long total = (long long)n.x * n.y * n.z;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int ax = (int)(t % n.x), r = (int)(t / n.x);
        const int by = r % n.y, cz = r / n.y;
        const int i = start.x + istep * ax, j = start.y + istep * by, k = DIM == 3 ? start.z + istep * cz : 1;
        float v;
        if (comp >= 0) v = interpolfld_one<DIM>(g, comp, a, (float)i, (float)j, (float)k) + add;
        else v = a[(i - 1) + g.sy * (j - 1) + g.sz * (k - 1)];
        out[t] = v;
    }
}

cudaError_t launch_output_sample(const Geom &g, int comp, const float *a, float add, const int start[3],
                                 const int n[3], int istep, float *out, cudaStream_t st) {
    const long long total = (long long)n[0] * n[1] * n[2];
    if (total <= 0) return cudaSuccess;
    const int3 s3 = make_int3(start[0], start[1], start[2]), n3 = make_int3(n[0], n[1], n[2]);
    if (g.dims == 3) k_output_sample<3><<<dgrid(total), 256, 0, st>>>(g, comp, a, add, s3, n3, istep, out);
    else k_output_sample<2><<<dgrid(total), 256, 0, st>>>(g, comp, a, add, s3, n3, istep, out);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// output_tot's particle sample (prtl.tot): particles with
// modulo(ind / 2, stride) = 0, compacted in the device's order
// ---------------------------------------------------------------------------
__global__ void k_prt_flag(Species sp, long long n, int stride, int *flag) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const int h = sp.ind[t] / 2;  // Fortran integer division: toward zero
        flag[t] = (sp.cell[t] >= 0 && ((h % stride) + stride) % stride == 0) ? 1 : 0;
    }
}

// vals: x + mxcum, y + mycum, z + mzcum, u, v, w, ch, gamma (cap each);
// ids: ind, proc (cap each)
template <int DIM>
__global__ void k_prt_write(Geom g, Params P, Species sp, long long n, const int *flag, const int *pos,
                            long long cap, float *vals, int *ids) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        if (!flag[t]) continue;
        const long long o = pos[t];
        float x, y, z;
        load_pos<DIM>(g, sp, t, x, y, z);
        const float u = sp.u[t], v = sp.v[t], w = sp.w[t];
        vals[o] = x + (float)P.mxcum;
        vals[cap + o] = y + (float)P.mycum;
        vals[2 * cap + o] = z + (float)P.mzcum;
        vals[3 * cap + o] = u;
        vals[4 * cap + o] = v;
        vals[5 * cap + o] = w;
        vals[6 * cap + o] = sp.ch[t];
        vals[7 * cap + o] = sqrtf(1.0f + (u * u + v * v + w * w));
        ids[o] = sp.ind[t];
        ids[cap + o] = sp.proc[t];
    }
}

cudaError_t launch_prt_flag(const Species &sp, long long n, int stride, int *flag, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    k_prt_flag<<<dgrid(n), 256, 0, st>>>(sp, n, stride, flag);
    return cudaGetLastError();
}

cudaError_t launch_prt_write(const Geom &g, const Params &P, const Species &sp, long long n, const int *flag,
                             const int *pos, long long cap, float *vals, int *ids, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (g.dims == 3) k_prt_write<3><<<dgrid(n), 256, 0, st>>>(g, P, sp, n, flag, pos, cap, vals, ids);
    else k_prt_write<2><<<dgrid(n), 256, 0, st>>>(g, P, sp, n, flag, pos, cap, vals, ids);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// flow-frame energy spectra per slice (save_spectrum_2d,
// code/output.F90:794-1249)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool spec_slice(const SpecGrid &sg, float x, float y, long long mxcum, long long mycum,
                                           int &sl) {
    const float fxb = (x + (float)mxcum - (float)sg.mxmin) / sg.dxslice + 1.0f;
    const float fyb = (y + (float)mycum - (float)sg.mymin) / sg.dyslice + 1.0f;
    if (!(fxb >= 1.0f && fyb >= 1.0f)) return false;
    const int xb = (int)fxb, yb = (int)fyb;
    if (xb > sg.nxb || yb > sg.nyb) return false;
    sl = (xb - 1) + sg.nxb * (yb - 1);
    return true;
}

// the spectrum weight of particle n: ch, or splitratio^(1 - splitlev) ch
__device__ __forceinline__ float spec_w(const SpecGrid &sg, const Species &sp, long long n) {
    if (!sg.split) return 1.0f;
    const int s = sp.splitlev[n];
    return (s >= 0 && s < 32) ? sg.wsplit[s] : powf(10.0f, 1.0f - (float)s);
}

// gamma range over every particle (starting from 1, as the reference)
__global__ void __launch_bounds__(256) k_spec_range(Species si, Species se, const long long *count,
                                                    unsigned *gmin, unsigned *gmax) {
    const long long n0 = count[0], n1 = count[1];
    float lo = 1.0f, hi = 1.0f;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n0 + n1;
         t += (long long)gridDim.x * blockDim.x) {
        const Species &sp = t < n0 ? si : se;
        const long long n = t < n0 ? t : t - n0;
        if (sp.cell[n] < 0) continue;
        const float u = sp.u[n], v = sp.v[n], w = sp.w[n];
        const float gam = sqrtf(1.0f + (u * u + v * v + w * w));
        lo = fminf(lo, gam);
        hi = fmaxf(hi, gam);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) {  // gamma >= 1 > 0: float order is integer order
        atomicMin(gmin, __float_as_uint(lo));
        atomicMax(gmax, __float_as_uint(hi));
    }
}

template <int DIM>
__global__ void __launch_bounds__(256) k_spec_means(Geom g, Params P, SpecGrid sg, Species sp, const long long *count,
                                                    double *acc) {
    const long long nsl = (long long)sg.nxb * sg.nyb;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < *count;
         n += (long long)gridDim.x * blockDim.x) {
        if (sp.cell[n] < 0 || (sg.ind_filter && sp.ind[n] <= 0)) continue;
        float x, y, z;
        load_pos<DIM>(g, sp, n, x, y, z);
        int sl;
        if (!spec_slice(sg, x, y, P.mxcum, P.mycum, sl)) continue;
        const float u = sp.u[n], v = sp.v[n], w = sp.w[n], ch = sp.ch[n];
        const float ws = spec_w(sg, sp, n);  // 1 unless split weights: products exact then
        const float gam = sqrtf(1.0f + (u * u + v * v + w * w));
        atomicAdd(acc + sl, (double)(ws * ch));
        atomicAdd(acc + nsl + sl, (double)((u / gam) * ws * ch));
        atomicAdd(acc + 2 * nsl + sl, (double)((v / gam) * ws * ch));
        atomicAdd(acc + 3 * nsl + sl, (double)((w / gam) * ws * ch));
    }
}

// slice means: the sums rounded to single, divided as the reference does
__global__ void k_spec_divide(long long nsl, double *acc, float *mean) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nsl;
         t += (long long)gridDim.x * blockDim.x) {
        const float nd = __double2float_rn(acc[t]);
        for (int c = 0; c < 3; c++) mean[c * nsl + t] = __double2float_rn(acc[(c + 1) * nsl + t]) / nd;
        for (int c = 0; c < 4; c++) acc[c * nsl + t] = 0.0;
    }
}

// per particle: the flow-frame gamma bin (and with spec_lab, the lab-frame
// one) gets the particle's weight
template <int DIM>
__global__ void __launch_bounds__(256) k_spec_bins(Geom g, Params P, SpecGrid sg, Species sp, const long long *count,
                                                   const float *mean, float lg0, float dgam, float *spec,
                                                   float *spec_lab) {
    const long long nsl = (long long)sg.nxb * sg.nyb;
    for (long long n = blockIdx.x * (long long)blockDim.x + threadIdx.x; n < *count;
         n += (long long)gridDim.x * blockDim.x) {
        if (sp.cell[n] < 0 || (sg.ind_filter && sp.ind[n] <= 0)) continue;
        float x, y, z;
        load_pos<DIM>(g, sp, n, x, y, z);
        int sl;
        if (!spec_slice(sg, x, y, P.mxcum, P.mycum, sl)) continue;
        const float u = sp.u[n], v = sp.v[n], w = sp.w[n], ch = sp.ch[n];
        const float wt = spec_w(sg, sp, n) * ch;
        const float gam = sqrtf(1.0f + (u * u + v * v + w * w));
        if (spec_lab) {
            const float fl = (log10_single(gam - 1.0f) - lg0) / dgam + 1.0f;
            if (fl >= 1.0f && fl < (float)sg.gambins + 1.0f) atomicAdd(spec_lab + sl + nsl * ((int)fl - 1), wt);
        }
        const float vx = mean[sl], vy = mean[nsl + sl], vz = mean[2 * nsl + sl];
        const float vr = sqrtf(vx * vx + vy * vy + vz * vz);
        const float gvr = 1.0f / sqrtf(1.0f - vr * vr);
        const float vr2 = vr * vr;
        const float up = -vx * gvr * gam + (1.0f + (gvr - 1.0f) * (vx * vx) / vr2) * u +
                         (gvr - 1.0f) * vx * vy / vr2 * v + (gvr - 1.0f) * vx * vz / vr2 * w;
        const float vp = -vy * gvr * gam + (gvr - 1.0f) * vx * vy / vr2 * u +
                         (1.0f + (gvr - 1.0f) * (vy * vy) / vr2) * v + (gvr - 1.0f) * vy * vz / vr2 * w;
        const float wp = -vz * gvr * gam + (gvr - 1.0f) * vx * vz / vr2 * u +
                         (gvr - 1.0f) * vy * vz / vr2 * v + (1.0f + (gvr - 1.0f) * (vz * vz) / vr2) * w;
        const float gp = sqrtf(1.0f + (up * up + vp * vp + wp * wp));
        const float fg = (log10_single(gp - 1.0f) - lg0) / dgam + 1.0f;
        if (!(fg >= 1.0f && fg < (float)sg.gambins + 1.0f)) continue;
        const int gbin = (int)fg;
        atomicAdd(spec + sl + nsl * (gbin - 1), wt);
    }
}

static int dgrid(long long n);

cudaError_t launch_spec_range(const Species *sp, const long long *count, long long hint, unsigned *gminmax,
                              cudaStream_t st) {
    k_spec_range<<<dgrid(hint), 256, 0, st>>>(sp[0], sp[1], count, gminmax, gminmax + 1);
    return cudaGetLastError();
}

cudaError_t launch_spec_species(const Geom &g, const Params &P, const SpecGrid &sg, const Species &sp,
                                const long long *count, long long hint, double *acc, float *mean, float lg0,
                                float dgam, float *spec, float *spec_lab, cudaStream_t st) {
    const long long nsl = (long long)sg.nxb * sg.nyb;
    if (g.dims == 3) {
        k_spec_means<3><<<dgrid(hint), 256, 0, st>>>(g, P, sg, sp, count, acc);
        k_spec_divide<<<dgrid(nsl), 256, 0, st>>>(nsl, acc, mean);
        k_spec_bins<3><<<dgrid(hint), 256, 0, st>>>(g, P, sg, sp, count, mean, lg0, dgam, spec, spec_lab);
    } else {
        k_spec_means<2><<<dgrid(hint), 256, 0, st>>>(g, P, sg, sp, count, acc);
        k_spec_divide<<<dgrid(nsl), 256, 0, st>>>(nsl, acc, mean);
        k_spec_bins<2><<<dgrid(hint), 256, 0, st>>>(g, P, sg, sp, count, mean, lg0, dgam, spec, spec_lab);
    }
    return cudaGetLastError();
}

static int dgrid(long long n) {
    long long b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > 152 * 8) b = 152 * 8;
    return (int)b;
}

cudaError_t launch_diag_particles(const DiagLaunch &d, cudaStream_t st) {
    const Geom &g = d.g;
    DiagArgs a;
    a.g = g;
    a.P = d.P;
    for (int s = 0; s < 2; s++) {
        a.sp[s] = d.sp[s];
        a.tstart[s] = d.tstart[s];
        a.mass[s] = d.mass[s];
    }
    a.rhofx = d.rhofx;
    a.acc = d.acc;
    a.status = d.status;
    a.only = d.only;
    const size_t smem = (size_t)g.wcells * 8;
    cudaError_t e = cudaSuccess;
#define TG_DL(D, O)                                                                                     \
    do {                                                                                                \
        e = cudaFuncSetAttribute(k_diag_particles<D, O>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                 (int)smem);                                                            \
        if (e != cudaSuccess) return e;                                                                 \
        k_diag_particles<D, O><<<g.ntiles, 256, smem, st>>>(a);                                         \
    } while (0)
    if (g.dims == 2 && g.order == 1) TG_DL(2, 1);
    else if (g.dims == 2 && g.order == 2) TG_DL(2, 2);
    else if (g.dims == 2 && g.order == 3) TG_DL(2, 3);
    else if (g.dims == 3 && g.order == 1) TG_DL(3, 1);
    else if (g.dims == 3 && g.order == 2) TG_DL(3, 2);
    else TG_DL(3, 3);
#undef TG_DL
    return cudaGetLastError();
}

cudaError_t launch_diag(const DiagLaunch &d, cudaStream_t st) {
    const Geom &g = d.g;
    cudaError_t e = cudaSuccess;
    if (d.particles && (e = launch_diag_particles(d, st)) != cudaSuccess) return e;
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int nx = g.mx - g.ng, ny = g.my - g.ng, nz = g.dims == 3 ? g.mz - g.ngz : 1;
    const long long n = (long long)nx * ny * nz;
    // the two FP64 scratch arrays hold the charge on its integer grid
    long long *cur = reinterpret_cast<long long *>(d.rho[0]), *nxt = reinterpret_cast<long long *>(d.rho[1]);
    k_rho_to_int<<<dgrid(n), 256, 0, st>>>(n, d.rhofx, cur, d.status);
    const int rg = rgrid(ny * nz);
    const size_t fsm = filter64_smem(g.dims);
    const dim3 fgrid((nx + TG_F64_TX - 1) / TG_F64_TX, (ny + TG_F64_TY(g.dims) - 1) / TG_F64_TY(g.dims),
                     (nz + TG_F64_TZ(g.dims) - 1) / TG_F64_TZ(g.dims));
    if (g.dims == 3)
        e = cudaFuncSetAttribute(k_filter_rho_pass<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsm);
    if (e != cudaSuccess) return e;
    for (int p = 0; p < d.ntimes; p++) {
        if (g.dims == 3) k_filter_rho_pass<3><<<fgrid, 256, fsm, st>>>(nx, ny, nz, cur, nxt);
        else k_filter_rho_pass<2><<<fgrid, 256, fsm, st>>>(nx, ny, nz, cur, nxt);
        long long *t = cur;
        cur = nxt;
        nxt = t;
    }
    const double inv = d.P.fx_inv / (double)(1LL << TG_RHO_SHIFT);
    if (g.dims == 3)
        k_diag_fields<3><<<rg, 256, 0, st>>>(g, d.f[0], d.f[1], d.f[2], d.f[3], d.f[4], d.f[5], cur, inv, d.acc);
    else
        k_diag_fields<2><<<rg, 256, 0, st>>>(g, d.f[0], d.f[1], d.f[2], d.f[3], d.f[4], d.f[5], cur, inv, d.acc);
    k_diag_finish<<<1, 32, 0, st>>>(d.acc, d.hist, d.hist_cap, d.counter);
    return cudaGetLastError();
}

}  // namespace tg

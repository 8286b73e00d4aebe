// Collisionless-shock hooks on the device (sm_103a, 2D): the left
// reflecting wall with its zigzag partial deposits (particle_bc_user,
// user_pu/user_shock_pu.F90:514-611; zigzag, code/particles.F90:550-669),
// the conductor and right-edge field reset (field_bc_user, :460-488) and
// the moving injector (inject_particles_user, :364-395, through
// inject_from_wall / inject_plasma_region, code/particles.F90:2439-2938).
//
// Random numbers: the reference draws from one Park-Miller stream
// (code/aux.F90:82-99), 13 draws per injected ion-electron pair in 2D with
// a magnetised plasma (3 for the position, 5 per Maxwell-Juttner momentum),
// plus one when a gamma draw comes out as exactly 1.0. Pair k of an
// injection therefore starts at seed * 16807^(13k) (mod 2^31 - 1) unless a
// redraw happened before it: every pair is drawn in parallel from that
// jump-ahead, the first pair that redrew is recorded, and the pairs after it
// are drawn again from the true state (sequentially in the finishing
// kernel, or in further parallel passes for large host-driven loads).
#include <cuda_runtime.h>

#include "tg_particles.cuh"

namespace tg {

__host__ __device__ inline long long mulmod31(long long a, long long b) {
    return (long long)(((unsigned long long)a * (unsigned long long)b) % 2147483647ULL);
}

__host__ __device__ inline long long powmod31(long long a, long long e) {
    long long r = 1;
    while (e > 0) {
        if (e & 1) r = mulmod31(r, a);
        a = mulmod31(a, a);
        e >>= 1;
    }
    return r;
}

// random(dseed): SEED = mod(16807 SEED, 2^31 - 1), SEED / 2^31 to single
__device__ __forceinline__ float pm_draw(long long &s) {
    s = (16807LL * s) % 2147483647LL;
    return __double2float_rn((double)s * 0x1p-31);
}

// sin and cos of a float: reduction by pi/2 in double (33-bit head of pi/2,
// so k * head is exact, and its tail), Taylor series to degree 17 on
// |r| <= pi/4, one rounding to single
__device__ __forceinline__ double sin_taylor(double r) {
    const double r2 = r * r;
    double t = 1.0 / 355687428096000.0;
    t = 1.0 / 1307674368000.0 - r2 * t;
    t = 1.0 / 6227020800.0 - r2 * t;
    t = 1.0 / 39916800.0 - r2 * t;
    t = 1.0 / 362880.0 - r2 * t;
    t = 1.0 / 5040.0 - r2 * t;
    t = 1.0 / 120.0 - r2 * t;
    t = 1.0 / 6.0 - r2 * t;
    return r - r * r2 * t;
}

__device__ __forceinline__ double cos_taylor(double r) {
    const double r2 = r * r;
    double t = 1.0 / 20922789888000.0;
    t = 1.0 / 87178291200.0 - r2 * t;
    t = 1.0 / 479001600.0 - r2 * t;
    t = 1.0 / 3628800.0 - r2 * t;
    t = 1.0 / 40320.0 - r2 * t;
    t = 1.0 / 720.0 - r2 * t;
    t = 1.0 / 24.0 - r2 * t;
    t = 0.5 - r2 * t;
    return 1.0 - r2 * t;
}

__device__ __forceinline__ void sincos_single(float x, float &sn, float &cs) {
    const double PIO2_HI = 0x1.921fb544p+0, PIO2_LO = 0x1.0b4611a626331p-34, TWO_OVER_PI = 0x1.45f306dc9c883p-1;
    const double xd = (double)x;
    const double k = rint(xd * TWO_OVER_PI);
    const double r = (xd - k * PIO2_HI) - k * PIO2_LO;
    const double s = sin_taylor(r), c = cos_taylor(r);
    const long long q = ((long long)k) & 3;
    double so, co;
    if (q == 0) { so = s; co = c; }
    else if (q == 1) { so = c; co = -s; }
    else if (q == 2) { so = -s; co = -c; }
    else { so = -c; co = s; }
    sn = __double2float_rn(so);
    cs = __double2float_rn(co);
}

// maxwell_dist (code/particles.F90:2176-2273), 2D build. The table is
// searched by bisection, which finds the same interval as the reference's
// linear scan (the table is non-decreasing and its intervals disjoint).
__device__ void maxwell(float gamma0, float cd, long long &seed, float &u, float &v, float &w, const float *gt,
                        const float *pt, float pcosthmult, int sigma_nonzero, bool &redrew) {
    const double pi = (double)3.1415927f;
    const float gamma0mag = fabsf(gamma0);
    const float gm = fmaxf(fabsf(gamma0), 1.0f);
    const float beta_drift = copysignf(sqrtf(1.0f - 1.0f / (gm * gm)), gamma0);
    float rannum = pm_draw(seed);
    if (rannum == 1.0f) {
        rannum = pm_draw(seed);
        redrew = true;
    }
    float gam;
    if (rannum >= pt[TG_PDF_SZ - 1]) {
        gam = gt[TG_PDF_SZ - 1];
    } else {
        int lo = 0, hi = TG_PDF_SZ - 1;  // pt[lo] <= rannum < pt[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (pt[mid] <= rannum) lo = mid;
            else hi = mid;
        }
        const int i = hi;  // 1-based interval index of the reference
        gam = gt[i - 1] + (gt[i] - gt[i - 1]) / (pt[i] - pt[i - 1]) * (rannum - pt[i - 1]);
    }
    float pcosth = (2.0f * pm_draw(seed) - 1.0f) * pcosthmult;
    if (sigma_nonzero) pcosth = 2.0f * pm_draw(seed) - 1.0f;
    const float pphi = __double2float_rn((double)(pm_draw(seed) * 2.0f) * pi);
    const float psinth = sqrtf(1.0f - pcosth * pcosth);
    const float v0t = cd * sqrtf(gam * (gam + 2.0f)) / (1.0f + gam);
    float sphi, cphi;
    sincos_single(pphi, sphi, cphi);
    const float ut1 = v0t * psinth * cphi;
    const float vt1 = v0t * psinth * sphi;
    const float wt1 = v0t * pcosth;
    float ptx = (1.0f + gam) * ut1;
    const float pty = (1.0f + gam) * vt1;
    const float ptz = (1.0f + gam) * wt1;
    const float X7 = pm_draw(seed);
    if (-beta_drift * ut1 / cd > X7) ptx = -ptx;
    const float px1 = (ptx + cd * beta_drift * (gam + 1.0f)) * gamma0mag;
    u = px1 / cd;
    v = pty / cd;
    w = ptz / cd;
}

__device__ __forceinline__ float effective_gamma_drift(float gdi) {
    return fabsf(gdi) < 1.0f ? copysignf(sqrtf(1.0f / (1.0f - gdi * gdi)), gdi) : gdi;
}

__device__ __forceinline__ void store_new(const Geom &g, const Species &sp, long long n, float x, float y, float z,
                                          float u, float v, float w, float ch, int ind, int *status) {
    int i, j, k;
    if (pos_cell<2>(g, x, y, z, i, j, k)) {
        store_pos<2>(g, sp, n, x, y, z, i, j, k);
    } else {
        sp.cell[n] = -1;
        atomicOr(status, ST_BOUNDS);
    }
    sp.u[n] = u;
    sp.v[n] = v;
    sp.w[n] = w;
    sp.ch[n] = ch;
    sp.ind[n] = ind;
    sp.proc[n] = 0;
    sp.splitlev[n] = 1;
}

// one ion-electron pair of inject_plasma_region (code/particles.F90:
// 2775-2860): position, ion momentum, electron at the same point
__device__ void inject_pair(const Geom &g, const ShockParams &K, const ShockState &S, float c, long long &seed,
                            int k, const Species *sp, bool write, int *status, bool &redrew) {
    const float x = S.minx + S.delta_x * pm_draw(seed);
    const float y = S.miny + S.delta_y * pm_draw(seed);
    const float z = S.minz + S.delta_z * pm_draw(seed);
    const float gd = effective_gamma_drift(K.gamma_drift);
    float ui, vi, wi, ue, ve, we;
    maxwell(gd, c, seed, ui, vi, wi, K.gt[0], K.pt[0], K.pcosthmult, K.sigma_nonzero, redrew);
    maxwell(gd, c, seed, ue, ve, we, K.gt[1], K.pt[1], K.pcosthmult, K.sigma_nonzero, redrew);
    if (!write) return;
    const float weight = S.weight;
    store_new(g, sp[0], S.base[0] + k, x, y, z, ui, vi, wi, weight, S.totalpartnum + 2 * k + 1, status);
    store_new(g, sp[1], S.base[1] + k, x, y, z, ue, ve, we, weight / 1.0f, S.totalpartnum + 2 * k + 2, status);
}

// ---------------------------------------------------------------------------
// injection plan (one thread): the injector's motion and slab
// (inject_particles_user + inject_from_wall) or an explicit region, then
// inject_plasma_region's extent and pair count
// ---------------------------------------------------------------------------
__global__ void k_inject_plan(Geom g, Params P, ShockParams K, ShockState *S, int mode, float x1, float x2,
                              float y1, float y2, float ppc, float weight, const long long *count,
                              long long maxhlf, int *status) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const float c = P.c;
    S->n = 0;
    S->k0 = 0;
    S->seed_k0 = S->seed;
    S->first_redraw = 0;
    if (mode == 0) {
        if (!K.inject) return;
        S->xinject2 = S->xinject2 + (double)(c * S->betainj);
        if (S->xinject2 > K.xinj_max) {
            S->xinject2 = K.xinj_max;
            S->betainj = 0.0f;
        }
        const float wall_speed = S->betainj;
        const float xw = (float)S->xinject2;
        const float beta_wall = fabsf(wall_speed) >= 1.0f
                                    ? copysignf(sqrtf(1.0f - 1.0f / (wall_speed * wall_speed)), wall_speed)
                                    : wall_speed;
        const float gd = K.gamma_drift;
        const float beta_inj = fabsf(gd) >= 1.0f ? copysignf(sqrtf(1.0f - 1.0f / (gd * gd)), gd) : gd;
        x1 = xw;
        x2 = xw + (beta_inj - beta_wall) * c;
        if (x2 < x1) {
            const float t = x1;
            x1 = x2;
            x2 = t;
        }
        y1 = K.y1;
        y2 = K.y2;
        ppc = K.ppc0;
        weight = K.weight;
        S->x2in = S->xinject2;  // read by the next lap's deposit
    }
    S->weight = weight;
    const int ng = g.ng, ngz = g.ngz;
    const long long iglob_min = (ng / 2 + 1) + P.mxcum, iglob_max = (g.mx - ng / 2) + P.mxcum;
    float minx = (float)(ng / 2 + 1), maxx = (float)(ng / 2 + 1);
    if (x1 < (float)iglob_min) minx = (float)(ng / 2 + 1);
    if (x2 < (float)iglob_min) maxx = (float)(ng / 2 + 1);
    if (x1 >= (float)iglob_max) minx = (float)(g.mx - ng / 2);
    if (x2 >= (float)iglob_max) maxx = (float)(g.mx - ng / 2);
    if (x1 >= (float)iglob_min && x1 < (float)iglob_max) minx = x1 - 1.0f * (float)P.mxcum;
    if (x2 >= (float)iglob_min && x2 < (float)iglob_max) maxx = x2 - 1.0f * (float)P.mxcum;
    const float delta_x = maxx - minx;
    const long long jglob_min = (ng / 2 + 1) + P.mycum, jglob_max = (g.my - ng / 2) + P.mycum;
    float miny = (float)(ng / 2 + 1), maxy = (float)(ng / 2 + 1);
    if (y1 < (float)jglob_min) miny = (float)(ng / 2 + 1);
    if (y2 < (float)jglob_min) maxy = (float)(ng / 2 + 1);
    if (y1 >= (float)jglob_max) miny = (float)(g.my - ng / 2);
    if (y2 >= (float)jglob_max) maxy = (float)(g.my - ng / 2);
    if (y1 >= (float)jglob_min && y1 < (float)jglob_max) miny = y1 - (float)P.mycum;
    if (y2 >= (float)jglob_min && y2 < (float)jglob_max) maxy = y2 - (float)P.mycum;
    float delta_y = maxy - miny;
    if (maxy == 0.0f || miny == 0.0f) {
        delta_y = 0.0f;
        maxy = 0.0f;
        miny = 0.0f;
    }
    const float maxz = 1.0f * (float)(ngz / 2 + 1) + 1.0f, minz = 1.0f * (float)(ngz / 2 + 1);
    const float delta_z = maxz - minz;
    float numps = (0.5f * ppc) * delta_z * delta_y * delta_x;
    long long seed = S->seed;
    if (numps < 10.0f) {
        if (numps != 0.0f) {
            // poisson (code/aux.F90:110-134)
            const double Lps = exp(-(double)numps);
            float kps = 0.0f;
            double pps = 1.0;
            while (pps >= Lps) {
                kps = kps + 1.0f;
                const float ups = pm_draw(seed);
                pps = pps * (double)ups;
            }
            numps = kps - 1.0f;
        } else {
            numps = 0.0f;
        }
    } else {
        numps = (float)(int)ceilf(numps);
    }
    int n = (int)numps;
    if (count[0] + n > maxhlf || count[1] + n > maxhlf) {
        atomicOr(status, ST_OVERFLOW);  // check_overflow_num would stop the run
        n = 0;
    }
    S->seed = seed;
    S->seed_k0 = seed;
    S->minx = minx;
    S->delta_x = delta_x;
    S->miny = miny;
    S->delta_y = delta_y;
    S->minz = minz;
    S->delta_z = delta_z;
    S->n = n;
    S->first_redraw = n;
    S->base[0] = count[0];
    S->base[1] = count[1];
}

// every pair of [k0, n) from the jump-ahead state
__global__ void __launch_bounds__(256) k_inject_pairs(Geom g, Params P, ShockParams K, ShockState *S, Species si,
                                                      Species se, int *status) {
    const ShockState s = *S;
    const Species sp[2] = {si, se};
    for (long long k = s.k0 + blockIdx.x * (long long)blockDim.x + threadIdx.x; k < s.n;
         k += (long long)gridDim.x * blockDim.x) {
        long long seed = mulmod31(s.seed_k0, powmod31(K.a13, k - s.k0));
        bool redrew = false;
        inject_pair(g, K, s, P.c, seed, (int)k, sp, true, status, redrew);
        if (redrew) atomicMin(&S->first_redraw, (int)k);
    }
}

// next pass starts after the first pair that redrew
__global__ void k_inject_fixup(Params P, ShockParams K, ShockState *S, Geom g) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int kf = S->first_redraw;
    if (kf >= S->n) return;
    long long seed = mulmod31(S->seed_k0, powmod31(K.a13, kf - S->k0));
    bool redrew = false;
    inject_pair(g, K, *S, P.c, seed, kf, nullptr, false, nullptr, redrew);
    S->k0 = kf + 1;
    S->seed_k0 = seed;
    S->first_redraw = S->n;
}

__global__ void k_inject_finish(Geom g, Params P, ShockParams K, ShockState *S, Species si, Species se,
                                long long *count, int *status) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const Species sp[2] = {si, se};
    const int n = S->n, kf = S->first_redraw;
    long long seed;
    if (kf < n) {
        seed = mulmod31(S->seed_k0, powmod31(K.a13, kf - S->k0));
        bool redrew = false;
        inject_pair(g, K, *S, P.c, seed, kf, sp, false, status, redrew);
        for (int k = kf + 1; k < n; k++) inject_pair(g, K, *S, P.c, seed, k, sp, true, status, redrew);
    } else {
        seed = mulmod31(S->seed_k0, powmod31(K.a13, n - S->k0));
    }
    S->seed = seed;
    S->totalpartnum += 2 * n;
    count[0] += n;
    count[1] += n;
}

// tile histogram of the injected particles (the sort that follows is told
// the counts of every particle); one species after the other, since the
// warp-aggregated increment merges lanes by tile index alone
__global__ void k_inject_count(Geom g, const ShockState *S, Species si, Species se, int *h0, int *h1) {
    const ShockState s = *S;
    for (int sidx = 0; sidx < 2; sidx++) {
        const Species &sp = sidx == 0 ? si : se;
        int *h = sidx == 0 ? h0 : h1;
        for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < s.n;
             k += (long long)gridDim.x * blockDim.x) {
            const int cell = sp.cell[s.base[sidx] + k];
            if (cell < 0) continue;
            int i, j, kk;
            cell_ijk(g, cell, i, j, kk);
            agg_inc(h, tile_of(g, i, j, kk));
        }
    }
}

// ---------------------------------------------------------------------------
// reflecting wall: particles behind the wall after the push
// ---------------------------------------------------------------------------
__global__ void k_wall_step(float c, float betawall, ShockState *S) {
    if (threadIdx.x == 0 && blockIdx.x == 0) S->walloc = S->walloc + (double)(betawall * c);
}

__global__ void __launch_bounds__(256) k_particle_bc(Geom g, Params P, ShockParams K, const ShockState *S,
                                                     Species si, Species se, const long long *count,
                                                     float *c0, float *c1, float *c2, unsigned long long *f0,
                                                     unsigned long long *f1, unsigned long long *f2, int *status,
                                                     int *dead) {
    WindowSink<true> sfx;
    WindowSink<false> s32;
    sfx.lo = s32.lo = nullptr;
    sfx.hi = s32.hi = nullptr;
    sfx.wx0 = s32.wx0 = 0;
    sfx.wy0 = s32.wy0 = 0;
    sfx.wz0 = s32.wz0 = 0;
    sfx.wx = s32.wx = 0;  // empty window: every addition goes to global memory
    sfx.wy = s32.wy = 0;
    sfx.wz = s32.wz = 0;
    sfx.wcells = s32.wcells = 0;
    float *gc[3] = {c0, c1, c2};
    unsigned long long *gf[3] = {f0, f1, f2};
    for (int a = 0; a < 3; a++) {
        sfx.gc[a] = s32.gc[a] = gc[a];
        sfx.gf[a] = s32.gf[a] = gf[a];
    }
    sfx.scale = s32.scale = P.fx_scale;
    sfx.g = s32.g = &g;
    sfx.status = s32.status = status;
    const double walloc = S->walloc;
    const long long n0 = count[0], n1 = count[1];
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n0 + n1;
         t += (long long)gridDim.x * blockDim.x) {
        const int s = t < n0 ? 0 : 1;
        const Species &sp = s == 0 ? si : se;
        const long long n = s == 0 ? t : t - n0;
        if (sp.cell[n] < 0) continue;
        float x, y, z;
        load_pos<2>(g, sp, n, x, y, z);
        if (!((double)(x + (float)P.mxcum) < walloc)) continue;
        float u = sp.u[n];
        const float v = sp.v[n], w = sp.w[n];
        const float q = sp.ch[n] * P.qs[s];
        bool keep;
        if (P.fixed) keep = wall_reflect(sfx, P.c, K.gammawall, K.betawall, walloc, P.mxcum, q, x, y, z, u, v, w);
        else keep = wall_reflect(s32, P.c, K.gammawall, K.betawall, walloc, P.mxcum, q, x, y, z, u, v, w);
        int i, j, k;
        if (keep && isfinite(x) && pos_cell<2>(g, x, y, z, i, j, k)) {
            store_pos<2>(g, sp, n, x, y, z, i, j, k);
            sp.u[n] = u;
        } else {
            sp.cell[n] = -1;  // removed (dropped by the next sort)
            *dead = 1;
        }
    }
}

// ---------------------------------------------------------------------------
// field_bc_user: conductor behind the wall, upstream fields at the right edge
// ---------------------------------------------------------------------------
__global__ void k_field_bc(Geom g, ShockParams K, float *ex, float *ey, float *ez, float *bx, float *by, float *bz) {
    const int nc = K.cond_i1 != K.cond_i2 ? K.cond_i2 - K.cond_i1 + 1 : 0;
    const int ne = K.edge_i1 != K.edge_i2 ? K.edge_i2 - K.edge_i1 + 1 : 0;
    const long long rows = (long long)g.my * g.mz;
    const long long total = (long long)(nc + ne) * rows;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int r = (int)(t % (nc + ne));
        const long long row = t / (nc + ne);
        const int j = (int)(row % g.my) + 1, k = (int)(row / g.my) + 1;
        if (r < nc) {
            const long long l = lin(g, K.cond_i1 + r, j, k);
            ey[l] = 0.0f;
            ez[l] = 0.0f;
        } else {
            const long long l = lin(g, K.edge_i1 + (r - nc), j, k);
            bx[l] = K.edge[3];
            by[l] = K.edge[4];
            bz[l] = K.edge[5];
            ex[l] = K.edge[0];
            ey[l] = K.edge[1];
            ez[l] = K.edge[2];
        }
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static int grid_for(long long n) {
    long long b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > 152 * 16) b = 152 * 16;
    return (int)b;
}

cudaError_t launch_field_bc(const Geom &g, const ShockParams &K, float *const *f, cudaStream_t st) {
    const int nc = K.cond_i1 != K.cond_i2 ? K.cond_i2 - K.cond_i1 + 1 : 0;
    const int ne = K.edge_i1 != K.edge_i2 ? K.edge_i2 - K.edge_i1 + 1 : 0;
    if (nc + ne == 0) return cudaSuccess;
    k_field_bc<<<grid_for((long long)(nc + ne) * g.my * g.mz), 256, 0, st>>>(g, K, f[0], f[1], f[2], f[3], f[4],
                                                                            f[5]);
    return cudaGetLastError();
}

cudaError_t launch_particle_bc(const Geom &g, const Params &P, const ShockParams &K, ShockState *S,
                               const Species *sp, const long long *count, long long hint, float *const *cur,
                               unsigned long long *const *fix, int *status, int *dead, cudaStream_t st) {
    if (!K.wall) return cudaSuccess;
    k_wall_step<<<1, 32, 0, st>>>(P.c, K.betawall, S);
    k_particle_bc<<<grid_for(hint), 256, 0, st>>>(g, P, K, S, sp[0], sp[1], count, cur[0], cur[1], cur[2],
                                                 fix[0], fix[1], fix[2], status, dead);
    return cudaGetLastError();
}

cudaError_t launch_wall_step(const Params &P, const ShockParams &K, ShockState *S, cudaStream_t st) {
    if (!K.wall) return cudaSuccess;
    k_wall_step<<<1, 32, 0, st>>>(P.c, K.betawall, S);
    return cudaGetLastError();
}

cudaError_t launch_inject_plan(const Geom &g, const Params &P, const ShockParams &K, ShockState *S, int mode,
                               float x1, float x2, float y1, float y2, float ppc, float weight,
                               const long long *count, long long maxhlf, int *status, cudaStream_t st) {
    k_inject_plan<<<1, 32, 0, st>>>(g, P, K, S, mode, x1, x2, y1, y2, ppc, weight, count, maxhlf, status);
    return cudaGetLastError();
}

cudaError_t launch_inject_pairs(const Geom &g, const Params &P, const ShockParams &K, ShockState *S,
                                const Species *sp, int grid, int *status, cudaStream_t st) {
    k_inject_pairs<<<grid, 256, 0, st>>>(g, P, K, S, sp[0], sp[1], status);
    return cudaGetLastError();
}

cudaError_t launch_inject_fixup(const Geom &g, const Params &P, const ShockParams &K, ShockState *S,
                                cudaStream_t st) {
    k_inject_fixup<<<1, 32, 0, st>>>(P, K, S, g);
    return cudaGetLastError();
}

cudaError_t launch_inject_finish(const Geom &g, const Params &P, const ShockParams &K, ShockState *S,
                                 const Species *sp, long long *count, int *const *hist, int grid, int *status,
                                 cudaStream_t st) {
    k_inject_finish<<<1, 32, 0, st>>>(g, P, K, S, sp[0], sp[1], count, status);
    if (hist) k_inject_count<<<grid, 256, 0, st>>>(g, S, sp[0], sp[1], hist[0], hist[1]);
    return cudaGetLastError();
}

}  // namespace tg

// Internal definitions of the GB300 TRISTAN-MP hot path (sm_103a).
//
// Floating point: every file is compiled with -fmad=false and IEEE division
// and square root, and every expression below is written in the reference
// Fortran's left-to-right order, so the mover and the field stencils round
// exactly as the reference does (one rounding per operation, no FMA).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tristan_gpu.h"

namespace tg {

// ---------------------------------------------------------------------------
// shape-function constants (code/particles.F90:235-248), single precision
// ---------------------------------------------------------------------------
#define TG_HALF 0.5f
#define TG_ONE 1.0f
#define TG_TWO 2.0f
#define TG_QUART 0.25f
#define TG_NINEIGHTH 1.125f
#define TG_THHALF 1.5f
#define TG_NEGONE (-1.0f)
#define TG_TWOTH 0x1.555556p-1f     // 2/3 rounded to single
#define TG_THIRD 0x1.555556p-2f     // 1/3
#define TG_SIXTH 0x1.555556p-3f     // 1/6
#define TG_NEGSIXTH (-0x1.555556p-3f)

// dynamic shared memory of a tile kernel: the deposit window (two 32-bit
// words per cell, three components) and the tile's field copy: in 2D the
// six field arrays over the window's cells, in 3D the primal copies (24 B
// per cell: a float4 and a float2 array) over the gather's reach, 16-byte
// aligned
__host__ __device__ inline size_t tile_window_bytes(int wcells) { return (size_t)6 * wcells * 4; }
__host__ __device__ inline size_t tile_fieldwin_offset(int wcells) { return (tile_window_bytes(wcells) + 15) & ~(size_t)15; }
__host__ __device__ inline size_t tile_smem_bytes(int dims, int wcells, int fwcells) {
    if (dims == 2) return 2 * tile_window_bytes(wcells);
    return fwcells > 0 ? tile_fieldwin_offset(wcells) + (size_t)24 * fwcells : tile_window_bytes(wcells);
}

// device status bits
enum : int32_t { ST_BOUNDS = 1, ST_NAN = 2, ST_OVERFLOW = 4, ST_WINDOW = 8, ST_CHARGE_GRID = 16 };

// ---------------------------------------------------------------------------
// Geometry of one domain (derived once at tg_init)
// ---------------------------------------------------------------------------
struct Geom {
    int dims, order;
    int mx, my, mz;
    int ng, ngz;
    long long lot;     // mx*my*mz
    long long sy, sz;  // strides: sy = mx, sz = mx*my
    int per[3];
    // particle position window kept by the periodic wrap
    float minx, maxx, miny, maxy, minz, maxz;
    // tiles: origin node of tile (0,0,0) and tile edges, tile counts
    int tx, ty, tz;
    int ox, oy, oz;
    int ntx, nty, ntz;
    int ntiles;
    // deposit window (per tile) = tile + [lo, hi] halo per axis
    int wlo, whi;  // halo below / above the tile, same on every axis
    int wx, wy, wz;
    int wcells;
    // 3D: the tile's copy of the primal fields over the gather's
    // reach (fw_lo cells below the tile, fwx x fwy x fwz cells), when two
    // CTAs per SM still fit beside the deposit window (fwcells = 0: none)
    int fw_lo, fwx, fwy, fwz, fwcells;
};

// particle storage: structure of arrays, cell index + in-cell offset
struct Species {
    int32_t *cell;  // 0-based linear index of node (aint x, aint y, aint z)
    float *ox, *oy;  // x - aint(x), y - aint(y)
    float *oz;       // 3D: z - aint(z); 2D: absolute z (not part of the cell)
    float *u, *v, *w, *ch;
    int32_t *ind, *proc, *splitlev;
};

struct Params {
    float c, corr, qm[2], qs[2];
    int external_fields;
    float ext[6];
    double x1in, x2in, y1in, y2in, z1in, z2in;
    long long mxcum, mycum, mzcum;
    int fixed;
    float fx_scale;    // 2^fx_shift
    double fx_inv;     // 2^-fx_shift
    int quirks;
};

// ---------------------------------------------------------------------------
// index helpers (1-based Fortran cell -> 0-based linear)
// ---------------------------------------------------------------------------
__host__ __device__ inline long long lin(const Geom &g, int i, int j, int k) {
    return (long long)(i - 1) + g.sy * (long long)(j - 1) + g.sz * (long long)(k - 1);
}

__device__ inline void cell_ijk(const Geom &g, int32_t cell, int &i, int &j, int &k) {
    int c = cell;
    i = c % g.mx + 1;
    c /= g.mx;
    if (g.dims == 3) {
        j = c % g.my + 1;
        k = c / g.my + 1;
    } else {
        j = c + 1;
        k = 1;
    }
}

// ---------------------------------------------------------------------------
// Shape factors. Weights of the NS nonzero slots starting at slot `base`
// (slot 3 = node aint(x)); identical forms in the movers and deposits
// (code/particles.F90:738-745, :928-1020, :1175-1277).
// ---------------------------------------------------------------------------
template <int ORDER> struct ShapeN;
template <> struct ShapeN<1> { static constexpr int NS = 2; static constexpr int U = 3; };
template <> struct ShapeN<2> { static constexpr int NS = 3; static constexpr int U = 5; };
template <> struct ShapeN<3> { static constexpr int NS = 4; static constexpr int U = 5; };

template <int ORDER>
__device__ __forceinline__ void shape(float d, float *w, int &base) {
    if (ORDER == 1) {
        w[0] = TG_ONE - d;
        w[1] = d;
        base = 3;
    } else if (ORDER == 2) {
        if (d <= TG_HALF) {
            float s2 = TG_HALF * (d * d - d + TG_QUART);
            float s4 = s2 + d;
            float s3 = TG_ONE - s4 - s2;
            w[0] = s2; w[1] = s3; w[2] = s4;
            base = 2;
        } else {
            float s3 = TG_NINEIGHTH - TG_THHALF * d + TG_HALF * d * d;
            float s5 = s3 - TG_ONE + d;
            float s4 = TG_ONE - s5 - s3;
            w[0] = s3; w[1] = s4; w[2] = s5;
            base = 3;
        }
    } else {
        if (d <= TG_HALF) {
            float s2 = TG_NEGSIXTH * (d - TG_ONE) * (d - TG_ONE) * (d - TG_ONE);
            float s3 = TG_TWOTH + TG_HALF * (d - TG_TWO) * d * d;
            float s5 = TG_SIXTH * d * d * d;
            float s4 = TG_ONE - s5 - s3 - s2;
            w[0] = s2; w[1] = s3; w[2] = s4; w[3] = s5;
        } else {
            float s5 = TG_SIXTH * d * d * d;
            float s4 = TG_TWOTH + TG_HALF * (TG_NEGONE - d) * (TG_ONE - d) * (TG_ONE - d);
            float s2 = TG_SIXTH * (TG_ONE - d) * (TG_ONE - d) * (TG_ONE - d);
            float s3 = TG_ONE - s5 - s4 - s2;
            w[0] = s2; w[1] = s3; w[2] = s4; w[3] = s5;
        }
        base = 2;
    }
}

// weight w[s - off] for static s, runtime off in [0, 2] (zero outside)
template <int NS>
__device__ __forceinline__ float pick(const float *w, int s, int off) {
    float r = 0.0f;
#pragma unroll
    for (int o = 0; o <= 2; o++) {
        int idx = s - o;
        if (idx >= 0 && idx < NS && off == o) r = w[idx];
    }
    return r;
}

// float -> fixed point for values known to be below 2^30 in magnitude (the
// deposit scale guarantees it for every contribution up to |q|); saturates
// otherwise and flags nothing: callers that cannot guarantee the bound use
// to_fixed
__device__ __forceinline__ long long to_fixed32(float x) { return (long long)__float2int_rn(x); }

// float -> int64 fixed point, round to nearest even (identical to llrintf);
// the int32 conversion is exact and cheap whenever the value fits
__device__ __forceinline__ long long to_fixed(float x) {
    if (fabsf(x) < 2147483520.0f) return (long long)__float2int_rn(x);
    return __float2ll_rn(x);
}

// a[i] for a runtime i in [0, N) without dynamic register indexing (which
// would spill the array to local memory): a chain of selects
template <int N>
__device__ __forceinline__ float sel(const float *a, int i) {
    float r = a[0];
#pragma unroll
    for (int k = 1; k < N; k++)
        if (i == k) r = a[k];
    return r;
}

// ---------------------------------------------------------------------------
// Fields seen by the particle kernels
// ---------------------------------------------------------------------------
struct FieldPtrs {
    const float *ex, *ey, *ez, *bx, *by, *bz;          // staggered Yee (2D gather)
    // primal copies (3D gather), interleaved: cell t holds (pex, pey, pez,
    // pbx) in prim[2t] and (pby, pbz, 0, 0) in prim[2t + 1], so a node's six
    // components come in two 16-byte loads
    const float4 *prim;
};

// A tile's copy of the six staggered 2D field arrays in shared memory over
// nodes x0 .. x0 + w - 1, y0 .. y0 + h - 1 (1-based), read by the gather of
// every particle whose nodes lie inside it. The components a gather node
// reads at one cell are paired: (ex, by) and (ey, bx) as float2 arrays,
// then ez and bz, w * h entries each.
struct FieldWin {
    const float *s;
    int x0, y0, w, h;
};

// A 3D tile's copy of the primal fields (FieldPtrs::prim) in shared memory
// over nodes x0 .. x0 + w - 1 (and y, z): (pex, pey, pez, pbx) in a float4
// array and (pby, pbz) in a float2 array, so that lanes at random cells
// spread over every bank (a 32-byte cell stride would start every 16-byte
// load on one of four bank groups)
struct FieldWin3 {
    const float4 *sa;
    const float2 *sb;
    int x0, y0, z0, w, h, d;
};

// ---------------------------------------------------------------------------
// Mover: shape-consistent gather + Boris + position advance, in absolute
// coordinates (mover_{1,2,3}ord, code/particles_movedeposit.F90:356-1271).
// The gather loops run over the dual shape's slot range (Q1 for order 2);
// 2D reads the staggered arrays with mixed weights, 3D the primal copies.
// ---------------------------------------------------------------------------
template <int DIM, int ORDER>
__device__ __forceinline__ void push_particle(const Geom &g, const FieldPtrs &f, const Params &P, float qm,
                                              float &x, float &y, float &z, float &u, float &v, float &w,
                                              const FieldWin *win = nullptr, const FieldWin3 *win3 = nullptr) {
    constexpr int NS = ShapeN<ORDER>::NS;
    const float c = P.c;
    const float cinv = 1.0f / c;
    int ip = (int)truncf(x);
    float dxp = x - (float)ip;
    int jp = (int)truncf(y);
    float dyp = y - (float)jp;
    int kp = (int)truncf(z);
    int id = (int)truncf(x - TG_HALF);
    float dxd = x - TG_HALF - (float)id;
    int jd = (int)truncf(y - TG_HALF);
    float dyd = y - TG_HALF - (float)jd;
    int kd = (int)truncf(z - TG_HALF);

    float wxp[NS], wyp[NS], wxd[NS], wyd[NS], wzp[NS], wzd[NS];
    int bxp, byp, bxd, byd, bzp = 0, bzd = 0;
    shape<ORDER>(dxp, wxp, bxp);
    shape<ORDER>(dyp, wyp, byp);
    shape<ORDER>(dxd, wxd, bxd);
    shape<ORDER>(dyd, wyd, byd);
    if (DIM == 3) {
        float dzp = z - (float)kp;
        float dzd = (z - TG_HALF) - (float)kd;
        shape<ORDER>(dzp, wzp, bzp);
        shape<ORDER>(dzd, wzd, bzd);
    }
    // primal weights seen through the dual slot range
    float axp[NS], ayp[NS], azp[NS];
#pragma unroll
    for (int r = 0; r < NS; r++) {
        if (ORDER == 2) {
            axp[r] = pick<NS>(wxp, r + 1, bxp - bxd + 1);
            ayp[r] = pick<NS>(wyp, r + 1, byp - byd + 1);
            if (DIM == 3) azp[r] = pick<NS>(wzp, r + 1, bzp - bzd + 1);
        } else {
            axp[r] = wxp[r];
            ayp[r] = wyp[r];
            if (DIM == 3) azp[r] = wzp[r];
        }
    }
    float ex0 = 0.0f, ey0 = 0.0f, ez0 = 0.0f, bx0 = 0.0f, by0 = 0.0f, bz0 = 0.0f;
    if (DIM == 3 && win3 && ip - 3 + bxd >= win3->x0 && ip - 4 + bxd + NS < win3->x0 + win3->w &&
        jp - 3 + byd >= win3->y0 && jp - 4 + byd + NS < win3->y0 + win3->h && kp - 3 + bzd >= win3->z0 &&
        kp - 4 + bzd + NS < win3->z0 + win3->d) {
        // every node in the tile's shared copy: the same loop on shared loads
        const int sy = win3->w, sz = win3->w * win3->h;
#pragma unroll 1
        for (int r3 = 0; r3 < NS; r3++) {
            const float az = sel<NS>(azp, r3);
#pragma unroll
            for (int r2 = 0; r2 < NS; r2++) {
                const int row = (ip - 3 + bxd - win3->x0) + sy * (jp - 3 + byd + r2 - win3->y0) +
                                sz * (kp - 3 + bzd + r3 - win3->z0);
                float sx = 0.0f, sy_ = 0.0f, sz_ = 0.0f, sbx = 0.0f, sby = 0.0f, sbz = 0.0f;
#pragma unroll
                for (int r1 = 0; r1 < NS; r1++) {
                    const int l = row + r1;
                    const float4 pa = win3->sa[l];
                    const float2 pb = win3->sb[l];
                    sx = sx + pa.x * axp[r1];
                    sy_ = sy_ + pa.y * axp[r1];
                    sz_ = sz_ + pa.z * axp[r1];
                    sbx = sbx + pa.w * axp[r1];
                    sby = sby + pb.x * axp[r1];
                    sbz = sbz + pb.y * axp[r1];
                }
                ex0 = ex0 + sx * ayp[r2] * az;
                ey0 = ey0 + sy_ * ayp[r2] * az;
                ez0 = ez0 + sz_ * ayp[r2] * az;
                bx0 = bx0 + sbx * ayp[r2] * az;
                by0 = by0 + sby * ayp[r2] * az;
                bz0 = bz0 + sbz * ayp[r2] * az;
            }
        }
    } else if (DIM == 3) {
        // planes rolled (code size), rows and columns unrolled
#pragma unroll 1
        for (int r3 = 0; r3 < NS; r3++) {
            const float az = sel<NS>(azp, r3);
#pragma unroll
            for (int r2 = 0; r2 < NS; r2++) {
                const int row = (ip - 3 + bxd - 1) + (int)g.sy * (jp - 3 + byd + r2 - 1) +
                                (int)g.sz * (kp - 3 + bzd + r3 - 1);
                float sx = 0.0f, sy = 0.0f, sz = 0.0f, sbx = 0.0f, sby = 0.0f, sbz = 0.0f;
#pragma unroll
                for (int r1 = 0; r1 < NS; r1++) {
                    const int l = row + r1;
                    const float4 pa = __ldg(f.prim + 2 * l), pb = __ldg(f.prim + 2 * l + 1);
                    sx = sx + pa.x * axp[r1];
                    sy = sy + pa.y * axp[r1];
                    sz = sz + pa.z * axp[r1];
                    sbx = sbx + pa.w * axp[r1];
                    sby = sby + pb.x * axp[r1];
                    sbz = sbz + pb.y * axp[r1];
                }
                ex0 = ex0 + sx * ayp[r2] * az;
                ey0 = ey0 + sy * ayp[r2] * az;
                ez0 = ez0 + sz * ayp[r2] * az;
                bx0 = bx0 + sbx * ayp[r2] * az;
                by0 = by0 + sby * ayp[r2] * az;
                bz0 = bz0 + sbz * ayp[r2] * az;
            }
        }
    } else if (win && id - 3 + bxd >= win->x0 && ip - 4 + bxd + NS < win->x0 + win->w &&
               jd - 3 + byd >= win->y0 && jp - 4 + byd + NS < win->y0 + win->h) {
        // every node in the tile's shared copy: the same loop on shared loads
        const int plane = win->w * win->h;
        const float2 *sxb = reinterpret_cast<const float2 *>(win->s), *syx = sxb + plane;
        const float *sez = reinterpret_cast<const float *>(syx + plane), *sbz = sez + plane;
#pragma unroll 1
        for (int r2 = 0; r2 < NS; r2++) {
            const int rowp = win->w * (jp - 3 + byd + r2 - win->y0);
            const int rowd = win->w * (jd - 3 + byd + r2 - win->y0);
            const float ay = sel<NS>(ayp, r2), wy = sel<NS>(wyd, r2);
#pragma unroll
            for (int r1 = 0; r1 < NS; r1++) {
                const int colp = ip - 3 + bxd + r1 - win->x0;
                const int cold = id - 3 + bxd + r1 - win->x0;
                const int lpp = colp + rowp, lpd = colp + rowd, ldp = cold + rowp, ldd = cold + rowd;
                const float2 eb = sxb[ldp], yb = syx[lpd];
                ex0 = ex0 + eb.x * wxd[r1] * ay;
                ey0 = ey0 + yb.x * axp[r1] * wy;
                ez0 = ez0 + sez[lpp] * axp[r1] * ay;
                bx0 = bx0 + yb.y * axp[r1] * wy;
                by0 = by0 + eb.y * wxd[r1] * ay;
                bz0 = bz0 + sbz[ldd] * wxd[r1] * wy;
            }
        }
    } else {
        // rows rolled (code size), columns unrolled
#pragma unroll 1
        for (int r2 = 0; r2 < NS; r2++) {
            const int rowp = (int)g.sy * (jp - 3 + byd + r2 - 1);
            const int rowd = (int)g.sy * (jd - 3 + byd + r2 - 1);
            const float ay = sel<NS>(ayp, r2), wy = sel<NS>(wyd, r2);
#pragma unroll
            for (int r1 = 0; r1 < NS; r1++) {
                const int colp = ip - 3 + bxd + r1 - 1;
                const int cold = id - 3 + bxd + r1 - 1;
                const int lpp = colp + rowp, lpd = colp + rowd, ldp = cold + rowp, ldd = cold + rowd;
                ex0 = ex0 + __ldg(f.ex + ldp) * wxd[r1] * ay;
                ey0 = ey0 + __ldg(f.ey + lpd) * axp[r1] * wy;
                ez0 = ez0 + __ldg(f.ez + lpp) * axp[r1] * ay;
                bx0 = bx0 + __ldg(f.bx + lpd) * axp[r1] * wy;
                by0 = by0 + __ldg(f.by + ldp) * wxd[r1] * ay;
                bz0 = bz0 + __ldg(f.bz + ldd) * wxd[r1] * wy;
            }
        }
    }
    (void)wzd;
    ex0 = 0.5f * ex0 * qm;
    ey0 = 0.5f * ey0 * qm;
    ez0 = 0.5f * ez0 * qm;
    bx0 = 0.5f * bx0 * qm * cinv;
    by0 = 0.5f * by0 * qm * cinv;
    bz0 = 0.5f * bz0 * qm * cinv;
    if (P.external_fields) {
        bx0 = bx0 + P.ext[3] * 0.5f * qm * cinv;
        by0 = by0 + P.ext[4] * 0.5f * qm * cinv;
        bz0 = bz0 + P.ext[5] * 0.5f * qm * cinv;
        ex0 = ex0 + P.ext[0] * 0.5f * qm;
        ey0 = ey0 + P.ext[1] * 0.5f * qm;
        ez0 = ez0 + P.ext[2] * 0.5f * qm;
    }
    // Boris rotation (code/particles_movedeposit.F90:564-583)
    float u0 = c * u + ex0;
    float v0 = c * v + ey0;
    float w0 = c * w + ez0;
    float gg = c / sqrtf(c * c + u0 * u0 + v0 * v0 + w0 * w0);
    bx0 = gg * bx0;
    by0 = gg * by0;
    bz0 = gg * bz0;
    float fr = 2.0f / (1.0f + bx0 * bx0 + by0 * by0 + bz0 * bz0);
    float u1 = (u0 + v0 * bz0 - w0 * by0) * fr;
    float v1 = (v0 + w0 * bx0 - u0 * bz0) * fr;
    float w1 = (w0 + u0 * by0 - v0 * bx0) * fr;
    u0 = u0 + v1 * bz0 - w1 * by0 + ex0;
    v0 = v0 + w1 * bx0 - u1 * bz0 + ey0;
    w0 = w0 + u1 * by0 - v1 * bx0 + ez0;
    u = u0 * cinv;
    v = v0 * cinv;
    w = w0 * cinv;
    gg = c / sqrtf(c * c + u0 * u0 + v0 * v0 + w0 * w0);
    x = x + u * gg * c;
    y = y + v * gg * c;
    z = z + w * gg * c;
}

// ---------------------------------------------------------------------------
// Periodic wrap / open-boundary keep test of deposit_particles' boundary
// loop for one rank (code/particles_movedeposit.F90:1546-1691).
// Returns false when the particle is discarded.
// ---------------------------------------------------------------------------
template <int DIM>
__device__ __forceinline__ bool wrap_particle(const Geom &g, const Params &P, float &x, float &y, float &z,
                                              double x2in) {
    const float midx = 0.5f * (g.maxx - g.minx), midy = 0.5f * (g.maxy - g.miny), midz = 0.5f * (g.maxz - g.minz);
    float perx = 0.0f, pery = 0.0f, perz = 0.0f;
    if (x < g.minx || x > g.maxx) perx = copysignf(midx, x - g.minx) + copysignf(midx, x - g.maxx);
    if (y < g.miny || y > g.maxy) pery = copysignf(midy, y - g.miny) + copysignf(midy, y - g.maxy);
    if (z < g.minz || z > g.maxz) perz = copysignf(midz, z - g.minz) + copysignf(midz, z - g.maxz);
    bool in = true;
    if (!g.per[0]) {
        float xg = x + (float)P.mxcum;
        in = ((double)xg > P.x1in) && ((double)xg < x2in);
    }
    if (!g.per[1] && in) {
        float yg = y + (float)P.mycum;
        in = ((double)yg > P.y1in) && ((double)yg < P.y2in);
    }
    if (DIM == 3 && !g.per[2] && in) {
        float zg = z + (float)P.mzcum;
        in = ((double)zg > P.z1in) && ((double)zg < P.z2in);
    }
    if (!in) {
        perx = 0.0f; pery = 0.0f; perz = 0.0f;
    }
    x = x - perx;
    y = y - pery;
    if (DIM == 3 && perz < 0.0f) perz = -((float)g.mz - 1.0f * (float)g.ngz);
    z = z - perz;
    return in;
}

// ---------------------------------------------------------------------------
// collisionless-shock hooks (tg_shock.cu)
// ---------------------------------------------------------------------------
#define TG_PDF_SZ 1000
// state the hooks update on the device (one per context)
struct ShockState {
    double xinject2, walloc, x2in;
    float betainj;
    int totalpartnum;
    long long seed;  // Park-Miller state, an integer in [1, 2^31 - 2]
    // the current injection: region, pairs, first pair of the running pass
    float minx, delta_x, miny, delta_y, minz, delta_z;
    int n, k0;
    long long seed_k0;
    int first_redraw;  // first pair of the pass whose gamma draw was redrawn (n: none)
    long long base[2];  // particle counts before the injection
    float weight;
};
// constants of the hooks
struct ShockParams {
    int wall, inject;
    float gammawall, betawall;
    int cond_i1, cond_i2, edge_i1, edge_i2;
    float edge[6];
    double xinj_max;
    float ppc0, gamma_drift, weight, y1, y2;
    float pcosthmult;
    int sigma_nonzero;
    const float *gt[2], *pt[2];  // Maxwell-Juttner tables of ions and electrons (device)
    long long a13;               // 16807^13 mod (2^31 - 1): one pair without redraws
};

// arguments of the tile kernel (particles sorted by tile)
struct TileArgs {
    Geom g;
    Params P;
    FieldPtrs f;
    Species sp[2];
    const int *tstart[2];  // [ntiles+1] per species
    int *newcount[2];      // histogram of the particles' new tiles
    float *cur[3];
    unsigned long long *fix[3];
    int *status;
    // shock hooks (null: none): the moving open boundary x2in and, with
    // wall != 0, the reflecting wall and its constants
    const ShockState *shock;
    int wall;
    float gammawall, betawall;
    // set to 1 when a particle is dropped on purpose (open boundary, wall),
    // so the host knows the next download must compact (null: not tracked)
    int *dead;
    // species of this launch: 0 both, 1 ions only, 2 electrons only
    int only;
};

// ---------------------------------------------------------------------------
// launchers (tg_particles.cu)
// ---------------------------------------------------------------------------
cudaError_t launch_tiles(const TileArgs &a, bool fixed, bool push, bool deposit, cudaStream_t st);
// the lap of the particles appended since the last tile sort (2D; injection)
cudaError_t launch_tail(const TileArgs &a, const long long *count, bool fixed, cudaStream_t st);
cudaError_t launch_push_flat(const Geom &g, const Params &P, const FieldPtrs &f, const Species &sp,
                             const long long *dcount, long long count, float qm, int *status, cudaStream_t st);
cudaError_t launch_tile_count(const Geom &g, const Species &sp, const long long *count, long long hint, int *hist,
                              cudaStream_t st);
cudaError_t launch_scan(int *hist, int *start, int *cursor, int n, long long *total, cudaStream_t st);
cudaError_t launch_scatter(const Geom &g, const Species &src, const Species &dst, const long long *count,
                           long long hint, const int *start, int *cursor, cudaStream_t st);
cudaError_t launch_gather(const Species &src, const Species &dst, const int *perm, long long count,
                          cudaStream_t st);
cudaError_t launch_reorder_keys(const Geom &g, const Species &sp, long long count, int *keys, int *idx,
                                cudaStream_t st);
cudaError_t launch_aos_to_soa(const Geom &g, const void *in, const Species &sp, long long count, int *status,
                              cudaStream_t st);
cudaError_t launch_soa_to_aos(const Geom &g, const Species &sp, void *out, long long count, cudaStream_t st);

// error text readable through tg_last_error(NULL) (tg_api.cu)
void tg_set_global_error(const char *msg);

// geometry and constants of one domain from its configuration (tg_api.cu);
// build_geom returns TG_OK or TG_ERR_ARG with the reason in err
int build_geom(const tg_config &c, Geom &g, char *err, size_t errlen);
void build_params(const tg_config &c, Params &P);
// one diagnostics record (16 doubles) as a tg_diag
void record_to_diag(const double *h, tg_diag *out);

// FP64 diagnostics (tg_diag.cu)
struct DiagLaunch {
    Geom g;
    Params P;
    Species sp[2];
    const int *tstart[2];
    float mass[2];
    const float *f[6];
    unsigned long long *rhofx;  // periodic interior, fixed point
    double *rho[2];             // periodic interior ping-pong (holds the int64 charge grid)
    double *acc;                // 16 accumulators
    double *hist;               // history ring [hist_cap][16]
    int hist_cap;
    unsigned long long *counter;
    int ntimes;
    int *status;
    bool particles;  // false: the particle pass already ran (part by part in a host-driven lap)
    int only;        // particle pass: 0 both species, 1 the ions only, 2 the electrons only
};
// the whole lap's diagnostics: particle pass (when d.particles), the
// charge's filter passes, the field reductions and the history record
cudaError_t launch_diag(const DiagLaunch &d, cudaStream_t st);
// the particle pass alone over d.sp / d.tstart (d.only selects the species)
cudaError_t launch_diag_particles(const DiagLaunch &d, cudaStream_t st);
// flow-frame spectra (save_spectrum_2d): the gamma range (two float bit
// patterns, seeded with 1.0), then per species slice means and the histogram
struct SpecGrid;
cudaError_t launch_spec_range(const Species *sp, const long long *count, long long hint, unsigned *gminmax,
                              cudaStream_t st);
cudaError_t launch_spec_species(const Geom &g, const Params &P, const SpecGrid &sg, const Species &sp,
                                const long long *count, long long hint, double *acc, float *mean, float lg0,
                                float dgam, float *spec, float *spec_lab, cudaStream_t st);
// output_tot's sampling: comp 0-5 interpolated E / B (plus add), comp < 0
// the array itself, at nodes start + istep (a, b, c), a < n[0] ... (tg_diag.cu)
cudaError_t launch_output_sample(const Geom &g, int comp, const float *a, float add, const int start[3],
                                 const int n[3], int istep, float *out, cudaStream_t st);
// output_tot's particle sample: flags of the selected particles, and the
// compacted values at the scanned positions (tg_diag.cu)
cudaError_t launch_prt_flag(const Species &sp, long long n, int stride, int *flag, cudaStream_t st);
cudaError_t launch_prt_write(const Geom &g, const Params &P, const Species &sp, long long n, const int *flag,
                             const int *pos, long long cap, float *vals, int *ids, cudaStream_t st);
// grid moments (meanq_fld_cur) into f3[0] (moment) and f3[1] (weight);
// num / den are zeroed FP64 scratch of g.lot cells, left zeroed
cudaError_t launch_moments(const Geom &g, const Params &P, const Species *sp, const long long *count, long long hint,
                           int kind, int idx, int idy, int idz, double *num, double *den, float *const *f3,
                           cudaStream_t st);

// shock hooks (tg_shock.cu)
cudaError_t launch_field_bc(const Geom &g, const ShockParams &K, float *const *f, cudaStream_t st);
// the wall's advance for this lap (before the push)
cudaError_t launch_wall_step(const Params &P, const ShockParams &K, ShockState *S, cudaStream_t st);
// wall advance and the wall over all particles (particle_bc_user alone)
cudaError_t launch_particle_bc(const Geom &g, const Params &P, const ShockParams &K, ShockState *S,
                               const Species *sp, const long long *count, long long hint, float *const *cur,
                               unsigned long long *const *fix, int *status, int *dead, cudaStream_t st);
// plan one injection: mode 0 = the moving injector's slab, 1 = the region
// (x1, x2, y1, y2) with ppc and weight
cudaError_t launch_inject_plan(const Geom &g, const Params &P, const ShockParams &K, ShockState *S, int mode,
                               float x1, float x2, float y1, float y2, float ppc, float weight,
                               const long long *count, long long maxhlf, int *status, cudaStream_t st);
// one parallel pass over the pairs [k0, n) of the plan
cudaError_t launch_inject_pairs(const Geom &g, const Params &P, const ShockParams &K, ShockState *S,
                                const Species *sp, int grid, int *status, cudaStream_t st);
// after a pass with a redraw at pair kf: the next pass starts at kf + 1
cudaError_t launch_inject_fixup(const Geom &g, const Params &P, const ShockParams &K, ShockState *S,
                                cudaStream_t st);
// finish: pairs after a remaining redraw sequentially, generator state,
// ind counter, particle counts; then (hist non-null) the new particles'
// tile histogram
cudaError_t launch_inject_finish(const Geom &g, const Params &P, const ShockParams &K, ShockState *S,
                                 const Species *sp, long long *count, int *const *hist, int grid, int *status,
                                 cudaStream_t st);

// launchers (tg_fields.cu); fields f[9] = ex ey ez bx by bz curx cury curz
enum GhostKind { GHOST_BC = 0, GHOST_FILTER = 1 };
cudaError_t launch_ghost(const Geom &g, float *a, float *b, float *c, GhostKind kind, cudaStream_t st);
cudaError_t launch_advance_b(const Geom &g, const Params &P, float *const *f, cudaStream_t st);
cudaError_t launch_advance_e(const Geom &g, const Params &P, float *const *f, cudaStream_t st);
cudaError_t launch_add_current(const Geom &g, float *const *f, cudaStream_t st);
cudaError_t launch_fold(const Geom &g, const Params &P, float *const *cur, cudaStream_t st);
// kernel launches of one launch_fold
int fold_launches(const Geom &g);
cudaError_t launch_filter_pass(const Geom &g, float *const *in, float *const *out, cudaStream_t st);
cudaError_t launch_primal(const Geom &g, float *const *f, float4 *prim, cudaStream_t st);
cudaError_t launch_fixed_to_float(const Geom &g, const Params &P, unsigned long long *const *fx, float *const *cur,
                                  cudaStream_t st);

}  // namespace tg

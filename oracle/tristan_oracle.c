/*
 * CPU oracle for the TRISTAN-MP per-step PIC hot path.
 *
 * TEST INFRASTRUCTURE ONLY (the oracle): the tests, the smoke check and
 * bench.py's CPU-baseline leg call it; the GPU product path never does.
 *
 * Each function restates one reference subroutine in the reference's own
 * floating-point operation order (left-to-right Fortran evaluation, one
 * rounding per operation, no FMA). File:line citations are to
 * mrowan137/tristan-mp-pu-master_densdecomp.
 *
 * Parity status: "parity unpinned" against reference outputs (the reference
 * ships no golden vectors and no Fortran toolchain exists to run it). The
 * restatement is pinned by an independent pure-Python transliteration
 * (tests/golden/make_golden.py, bit-exact agreement required) and by
 * physics known-answer tests (tests/test_oracle_physics.py).
 *
 * Choices where the reference is undefined, stated once here:
 *  - densdecomp_1ord never initialises curx_add_prev / cury_add_prevs
 *    (code/particles.F90:717-732); they are taken as 0 here, as the 2nd and
 *    3rd order routines initialise them (:907-910, :1155-1158).
 *  - pind is never zeroed for ions before first use (code/particles.F90:319,
 *    particles_movedeposit.F90:1544 commented out); it is taken as 0.
 *  - the shape-mismatched copy at code/fieldboundaries.F90:1938 folds the
 *    full nghost/2+1 rows of cury by default; TO_QUIRK_Q5_LHS reproduces the
 *    left-hand-side-extent reading instead.
 */
#include "tristan_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* shape-function constants as code/particles.F90:235-248 computes them in
   single precision */
#define HALF 0.5f
#define ONE 1.0f
#define TWO 2.0f
#define QUART 0.25f
#define NINEIGHTH 1.125f
#define THHALF 1.5f
#define NEGONE (-1.0f)
static const float TWOTH = 2.0f / 3.0f;
static const float THIRD = 1.0f / 3.0f;
static const float SIXTH = 1.0f / 6.0f;
static const float NEGSIXTH = -(1.0f / 6.0f);

int to_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

int64_t to_lot(const to_state *s) { return (int64_t)s->mx * s->my * s->mz; }

/* 0-based linear index of the 1-based Fortran cell (i,j,k) */
static inline int64_t L3(const to_state *s, int64_t i, int64_t j, int64_t k)
{
    return (i - 1) + (int64_t)s->mx * ((j - 1) + (int64_t)s->my * (k - 1));
}

/* ------------------------------------------------------------------------
 * Shape factors. S is indexed by the reference's slot number 1..6; slot 3
 * holds the weight of node aint(x). `off` is the slot shift used by the
 * deposit for the new position (Sx2(3+shifti) ...). Sets [*mn,*mxs].
 * Orders: code/particles.F90:738-745 (1st), :928-1020 (2nd),
 * :1175-1277 (3rd); identical forms in the movers
 * (code/particles_movedeposit.F90:447-468, :709-790, :1035-1128).
 * --------------------------------------------------------------------- */
static void shape(int order, float d, float *S, int off, int *mn, int *mxs)
{
    if (order == 1) {
        S[3 + off] = ONE - d;
        S[4 + off] = d;
        *mn = 3 + off;
        *mxs = 4 + off;
    } else if (order == 2) {
        if (d <= HALF) {
            S[2 + off] = HALF * (d * d - d + QUART);
            S[4 + off] = S[2 + off] + d;
            S[3 + off] = ONE - S[4 + off] - S[2 + off];
            *mn = 2 + off;
            *mxs = 4 + off;
        } else if (d > HALF) {
            S[3 + off] = NINEIGHTH - THHALF * d + HALF * d * d;
            S[5 + off] = S[3 + off] - ONE + d;
            S[4 + off] = ONE - S[5 + off] - S[3 + off];
            *mn = 3 + off;
            *mxs = 5 + off;
        }
    } else {
        if (d <= HALF) {
            S[2 + off] = NEGSIXTH * (d - ONE) * (d - ONE) * (d - ONE);
            S[3 + off] = TWOTH + HALF * (d - TWO) * d * d;
            S[5 + off] = SIXTH * d * d * d;
            S[4 + off] = ONE - S[5 + off] - S[3 + off] - S[2 + off];
        } else if (d > HALF) {
            S[5 + off] = SIXTH * d * d * d;
            S[4 + off] = TWOTH + HALF * (NEGONE - d) * (ONE - d) * (ONE - d);
            S[2 + off] = SIXTH * (ONE - d) * (ONE - d) * (ONE - d);
            S[3 + off] = ONE - S[5 + off] - S[4 + off] - S[2 + off];
        }
        *mn = 2 + off;
        *mxs = 5 + off;
    }
}

/* ------------------------------------------------------------------------
 * Movers: mover_1ord / mover_2ord / mover_3ord
 * (code/particles_movedeposit.F90:356-610, :619-933, :943-1271).
 * The loop ranges are the dual shape's (the dual assignment overwrites the
 * primal iter*min/max), which truncates the 2nd-order primal weights (Q1).
 * 2D gathers from the staggered Yee arrays with mixed primal/dual weights;
 * 3D gathers from primal-averaged copies with primal weights (Q2, Q3).
 * --------------------------------------------------------------------- */
typedef struct {
    float *ex_p, *ey_p, *ez_p, *bx_p, *by_p, *bz_p;
} primal_fields;

/* primal grids, code/particles_movedeposit.F90:395-404 (cshift wraps over
   the full local array, ghosts included) */
static void make_primal(const to_state *s, primal_fields *pf)
{
    int64_t lot = to_lot(s);
    int mx = s->mx, my = s->my, mz = s->mz;
    pf->ex_p = malloc(sizeof(float) * lot);
    pf->ey_p = malloc(sizeof(float) * lot);
    pf->ez_p = malloc(sizeof(float) * lot);
    pf->bx_p = malloc(sizeof(float) * lot);
    pf->by_p = malloc(sizeof(float) * lot);
    pf->bz_p = malloc(sizeof(float) * lot);
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= mz; k++) {
        int km = (k == 1) ? mz : k - 1;
        for (int j = 1; j <= my; j++) {
            int jm = (j == 1) ? my : j - 1;
            for (int i = 1; i <= mx; i++) {
                int im = (i == 1) ? mx : i - 1;
                int64_t l = L3(s, i, j, k);
                pf->ex_p[l] = 0.5f * (s->ex[l] + s->ex[L3(s, im, j, k)]);
                pf->ey_p[l] = 0.5f * (s->ey[l] + s->ey[L3(s, i, jm, k)]);
                pf->ez_p[l] = 0.5f * (s->ez[l] + s->ez[L3(s, i, j, km)]);
                pf->bx_p[l] = 0.5f * (s->bx[l] + s->bx[L3(s, i, jm, k)]);
                pf->by_p[l] = 0.5f * (s->by[l] + s->by[L3(s, im, j, k)]);
                pf->bz_p[l] = 0.5f * (0.5f * (s->bz[l] + s->bz[L3(s, im, j, k)]) +
                                      0.5f * (s->bz[L3(s, i, jm, k)] + s->bz[L3(s, im, jm, k)]));
            }
        }
    }
}

static void free_primal(primal_fields *pf)
{
    free(pf->ex_p); free(pf->ey_p); free(pf->ez_p);
    free(pf->bx_p); free(pf->by_p); free(pf->bz_p);
}

static void push_one(const to_state *s, const primal_fields *pf, to_particle *pp, float qm)
{
    const float c = s->c;
    const float cinv = 1.0f / c;
    const int order = s->order;
    const int64_t iy = s->mx, iz = (int64_t)s->mx * s->my;
    float Sxp[8], Syp[8], Szp[8], Sxd[8], Syd[8], Szd[8];
    int i1min, i1max, i2min, i2max, i3min = 0, i3max = -1;
    memset(Sxp, 0, sizeof Sxp); memset(Syp, 0, sizeof Syp); memset(Szp, 0, sizeof Szp);
    memset(Sxd, 0, sizeof Sxd); memset(Syd, 0, sizeof Syd); memset(Szd, 0, sizeof Szd);

    const float x = pp->x, y = pp->y, z = pp->z;
    int ip = (int)truncf(x);
    float dxp = x - (float)ip;
    int jp = (int)truncf(y);
    float dyp = y - (float)jp;
    int kp = (int)truncf(z);
    int id = (int)truncf(x - HALF);
    float dxd = x - HALF - (float)id;
    int jd = (int)truncf(y - HALF);
    float dyd = y - HALF - (float)jd;
    int kd = (int)truncf(z - HALF);
    float dzp = 0.0f, dzd = 0.0f;
    if (s->dims == 3) {
        dzp = z - (float)kp;
        dzd = (z - HALF) - (float)kd;
    }
    int dmy;
    /* primal first, then dual: the dual's ranges are the ones kept */
    shape(order, dxp, Sxp, 0, &i1min, &i1max);
    shape(order, dyp, Syp, 0, &i2min, &i2max);
    if (s->dims == 3) shape(order, dzp, Szp, 0, &i3min, &i3max);
    shape(order, dxd, Sxd, 0, &i1min, &i1max);
    shape(order, dyd, Syd, 0, &i2min, &i2max);
    if (s->dims == 3) shape(order, dzd, Szd, 0, &i3min, &i3max);
    (void)dmy;

    float ex0 = 0.0f, ey0 = 0.0f, ez0 = 0.0f, bx0 = 0.0f, by0 = 0.0f, bz0 = 0.0f;
    if (s->dims == 3) {
        for (int it3 = i3min; it3 <= i3max; it3++) {
            for (int it2 = i2min; it2 <= i2max; it2++) {
                int64_t jj = jp - 3 + it2, kk = kp - 3 + it3;
                float sx = 0.0f, sy = 0.0f, sz = 0.0f, sbx = 0.0f, sby = 0.0f, sbz = 0.0f;
                for (int it1 = i1min; it1 <= i1max; it1++) {
                    int64_t l = L3(s, ip - 3 + it1, jj, kk);
                    sx = sx + pf->ex_p[l] * Sxp[it1];
                    sy = sy + pf->ey_p[l] * Sxp[it1];
                    sz = sz + pf->ez_p[l] * Sxp[it1];
                    sbx = sbx + pf->bx_p[l] * Sxp[it1];
                    sby = sby + pf->by_p[l] * Sxp[it1];
                    sbz = sbz + pf->bz_p[l] * Sxp[it1];
                }
                ex0 = ex0 + sx * Syp[it2] * Szp[it3];
                ey0 = ey0 + sy * Syp[it2] * Szp[it3];
                ez0 = ez0 + sz * Syp[it2] * Szp[it3];
                bx0 = bx0 + sbx * Syp[it2] * Szp[it3];
                by0 = by0 + sby * Syp[it2] * Szp[it3];
                bz0 = bz0 + sbz * Syp[it2] * Szp[it3];
            }
        }
    } else {
        for (int it2 = i2min; it2 <= i2max; it2++) {
            for (int it1 = i1min; it1 <= i1max; it1++) {
                /* 1-based linear indices as the reference builds them */
                int64_t lpp = (ip - 3 + it1) + iy * (jp - 3 + it2 - 1);
                int64_t lpd = (ip - 3 + it1) + iy * (jd - 3 + it2 - 1);
                int64_t ldp = (id - 3 + it1) + iy * (jp - 3 + it2 - 1);
                int64_t ldd = (id - 3 + it1) + iy * (jd - 3 + it2 - 1);
                ex0 = ex0 + s->ex[ldp - 1] * Sxd[it1] * Syp[it2];
                ey0 = ey0 + s->ey[lpd - 1] * Sxp[it1] * Syd[it2];
                ez0 = ez0 + s->ez[lpp - 1] * Sxp[it1] * Syp[it2];
                bx0 = bx0 + s->bx[lpd - 1] * Sxp[it1] * Syd[it2];
                by0 = by0 + s->by[ldp - 1] * Sxd[it1] * Syp[it2];
                bz0 = bz0 + s->bz[ldd - 1] * Sxd[it1] * Syd[it2];
            }
        }
    }
    (void)iz;

    ex0 = 0.5f * ex0 * qm;
    ey0 = 0.5f * ey0 * qm;
    ez0 = 0.5f * ez0 * qm;
    bx0 = 0.5f * bx0 * qm * cinv;
    by0 = 0.5f * by0 * qm * cinv;
    bz0 = 0.5f * bz0 * qm * cinv;

    if (s->external_fields) {
        bx0 = bx0 + s->ext[3] * 0.5f * qm * cinv;
        by0 = by0 + s->ext[4] * 0.5f * qm * cinv;
        bz0 = bz0 + s->ext[5] * 0.5f * qm * cinv;
        ex0 = ex0 + s->ext[0] * 0.5f * qm;
        ey0 = ey0 + s->ext[1] * 0.5f * qm;
        ez0 = ez0 + s->ext[2] * 0.5f * qm;
    }

    /* Boris, code/particles_movedeposit.F90:564-583 */
    float u0 = c * pp->u + ex0;
    float v0 = c * pp->v + ey0;
    float w0 = c * pp->w + ez0;
    float g = c / sqrtf(c * c + u0 * u0 + v0 * v0 + w0 * w0);
    bx0 = g * bx0;
    by0 = g * by0;
    bz0 = g * bz0;
    float f = 2.0f / (1.0f + bx0 * bx0 + by0 * by0 + bz0 * bz0);
    float u1 = (u0 + v0 * bz0 - w0 * by0) * f;
    float v1 = (v0 + w0 * bx0 - u0 * bz0) * f;
    float w1 = (w0 + u0 * by0 - v0 * bx0) * f;
    u0 = u0 + v1 * bz0 - w1 * by0 + ex0;
    v0 = v0 + w1 * bx0 - u1 * bz0 + ey0;
    w0 = w0 + u1 * by0 - v1 * bx0 + ez0;
    pp->u = u0 * cinv;
    pp->v = v0 * cinv;
    pp->w = w0 * cinv;
    /* position advance, :602-606 */
    g = c / sqrtf(c * c + u0 * u0 + v0 * v0 + w0 * w0);
    pp->x = pp->x + pp->u * g * c;
    pp->y = pp->y + pp->v * g * c;
    pp->z = pp->z + pp->w * g * c;
}

void to_mover(to_state *s, int64_t n1, int64_t n2, float qm)
{
    primal_fields pf = {0};
    if (s->dims == 3) make_primal(s, &pf);
#pragma omp parallel for schedule(static)
    for (int64_t n = n1; n < n2; n++) push_one(s, &pf, &s->p[n], qm);
    if (s->dims == 3) free_primal(&pf);
}

/* code/particles_movedeposit.F90:63-88 */
void to_move_particles(to_state *s)
{
    to_mover(s, 0, s->ions, s->qmi);
    to_mover(s, s->maxhlf, s->maxhlf + s->lecs, s->qme);
}

/* ------------------------------------------------------------------------
 * Esirkepov deposit, densdecomp_{1,2,3}ord (code/particles.F90:678-1358).
 * The x carry (curx_add_prev) is not reset between rows, and the y carries
 * (cury_add_prevs) not between planes (Q4). `acc` receives each addition:
 * FP32 into cur*, or int64 fixed point.
 * --------------------------------------------------------------------- */
typedef struct {
    float *cx, *cy, *cz;
    int64_t *fx, *fy, *fz;
    float scale;
    int64_t lot;
    int fixed;
} dep_target;

static inline void dep_add(const dep_target *t, int comp, int64_t l, float v)
{
    if (l < 0 || l >= t->lot) return; /* the reference writes out of bounds */
    if (t->fixed) {
        int64_t q = llrintf(v * t->scale);
        if (comp == 0) t->fx[l] += q;
        else if (comp == 1) t->fy[l] += q;
        else t->fz[l] += q;
    } else {
        if (comp == 0) t->cx[l] = t->cx[l] + v;
        else if (comp == 1) t->cy[l] = t->cy[l] + v;
        else t->cz[l] = t->cz[l] + v;
    }
}

static void densdecomp(const to_state *s, const dep_target *t, float x2, float y2, float z2,
                       float x1, float y1, float z1, float q)
{
    const int order = s->order;
    const int64_t iy = s->mx, iz = (int64_t)s->mx * s->my;
    float Sx1[8], Sy1[8], Sx2[8], Sy2[8], Sz1[8], Sz2[8];
    float cury_adds[8], cury_add_prevs[8], curz_adds[8][8], curz_add_prevs[8][8];
    float curx_add = 0.0f, curx_add_prev = 0.0f, curz_add = 0.0f;
    memset(Sx1, 0, sizeof Sx1); memset(Sx2, 0, sizeof Sx2);
    memset(Sy1, 0, sizeof Sy1); memset(Sy2, 0, sizeof Sy2);
    memset(Sz1, 0, sizeof Sz1); memset(Sz2, 0, sizeof Sz2);
    memset(cury_adds, 0, sizeof cury_adds); memset(cury_add_prevs, 0, sizeof cury_add_prevs);
    memset(curz_adds, 0, sizeof curz_adds); memset(curz_add_prevs, 0, sizeof curz_add_prevs);

    int i1 = (int)truncf(x1), i2 = (int)truncf(x2);
    int j1 = (int)truncf(y1), j2 = (int)truncf(y2);
    int k1 = (int)truncf(z1), k2 = (int)truncf(z2);
    int shifti = i2 - i1, shiftj = j2 - j1, shiftk = k2 - k1;
    float dx1 = x1 - truncf(x1), dy1 = y1 - truncf(y1);
    float dx2 = x2 - truncf(x2), dy2 = y2 - truncf(y2);
    float dz1 = z1 - truncf(z1), dz2 = z2 - truncf(z2);
    float deltaz = z2 - z1;
    if (s->dims == 2) { k1 = 1; k2 = 1; shiftk = 0; }
    (void)k2;

    int x1mn, x1mx, x2mn, x2mx, y1mn, y1mx, y2mn, y2mx, z1mn = 0, z1mx = 0, z2mn = 0, z2mx = 0;
    shape(order, dx1, Sx1, 0, &x1mn, &x1mx);
    shape(order, dy1, Sy1, 0, &y1mn, &y1mx);
    if (s->dims == 3) shape(order, dz1, Sz1, 0, &z1mn, &z1mx);
    shape(order, dx2, Sx2, shifti, &x2mn, &x2mx);
    shape(order, dy2, Sy2, shiftj, &y2mn, &y2mx);
    if (s->dims == 3) shape(order, dz2, Sz2, shiftk, &z2mn, &z2mx);
    int xmn = x1mn < x2mn ? x1mn : x2mn, xmx = x1mx > x2mx ? x1mx : x2mx;
    int ymn = y1mn < y2mn ? y1mn : y2mn, ymx = y1mx > y2mx ? y1mx : y2mx;

    if (s->dims == 3) {
        int zmn = z1mn < z2mn ? z1mn : z2mn, zmx = z1mx > z2mx ? z1mx : z2mx;
        for (int it2 = zmn; it2 <= zmx; it2++) {
            for (int it1 = ymn; it1 <= ymx; it1++) {
                for (int it = xmn; it <= xmx; it++) {
                    int64_t l2 = (i1 - 3 + it) + (int64_t)(j1 - 3 + it1 - 1) * iy +
                                 (int64_t)(k1 - 3 + it2 - 1) * iz;
                    curx_add = q * ((Sx2[it] - Sx1[it]) *
                                    (Sy1[it1] * Sz1[it2] + HALF * (Sy2[it1] - Sy1[it1]) * Sz1[it2] +
                                     HALF * Sy1[it1] * (Sz2[it2] - Sz1[it2]) +
                                     THIRD * (Sy2[it1] - Sy1[it1]) * (Sz2[it2] - Sz1[it2]))) +
                               curx_add_prev;
                    cury_adds[it] = q * ((Sy2[it1] - Sy1[it1]) *
                                         (Sx1[it] * Sz1[it2] + HALF * (Sx2[it] - Sx1[it]) * Sz1[it2] +
                                          HALF * Sx1[it] * (Sz2[it2] - Sz1[it2]) +
                                          THIRD * (Sx2[it] - Sx1[it]) * (Sz2[it2] - Sz1[it2]))) +
                                    cury_add_prevs[it];
                    curz_adds[it][it1] = q * ((Sz2[it2] - Sz1[it2]) *
                                              (Sx1[it] * Sy1[it1] + HALF * (Sx2[it] - Sx1[it]) * Sy1[it1] +
                                               HALF * Sx1[it] * (Sy2[it1] - Sy1[it1]) +
                                               THIRD * (Sx2[it] - Sx1[it]) * (Sy2[it1] - Sy1[it1]))) +
                                         curz_add_prevs[it][it1];
                    dep_add(t, 0, l2 - 1, curx_add);
                    dep_add(t, 1, l2 - 1, cury_adds[it]);
                    dep_add(t, 2, l2 - 1, curz_adds[it][it1]);
                    curx_add_prev = curx_add;
                }
                curx_add = 0.0f;
                memcpy(cury_add_prevs, cury_adds, sizeof cury_adds);
                memset(cury_adds, 0, sizeof cury_adds);
            }
            memcpy(curz_add_prevs, curz_adds, sizeof curz_adds);
            memset(curz_adds, 0, sizeof curz_adds);
        }
    } else {
        for (int it1 = ymn; it1 <= ymx; it1++) {
            for (int it = xmn; it <= xmx; it++) {
                int64_t l2 = (i1 - 3 + it) + (int64_t)(j1 - 3 + it1 - 1) * iy;
                curx_add = q * ((Sx2[it] - Sx1[it]) * (Sy1[it1] + HALF * (Sy2[it1] - Sy1[it1]))) +
                           curx_add_prev;
                cury_adds[it] = q * ((Sy2[it1] - Sy1[it1]) * (Sx1[it] + HALF * (Sx2[it] - Sx1[it]))) +
                                cury_add_prevs[it];
                curz_add = -(q * deltaz *
                             (Sx1[it] * Sy1[it1] + HALF * (Sx2[it] - Sx1[it]) * Sy1[it1] +
                              HALF * Sx1[it] * (Sy2[it1] - Sy1[it1]) +
                              THIRD * (Sx2[it] - Sx1[it]) * (Sy2[it1] - Sy1[it1])));
                dep_add(t, 0, l2 - 1, curx_add);
                dep_add(t, 1, l2 - 1, cury_adds[it]);
                dep_add(t, 2, l2 - 1, curz_add);
                curx_add_prev = curx_add;
            }
            curx_add = 0.0f;
            memcpy(cury_add_prevs, cury_adds, sizeof cury_adds);
            memset(cury_adds, 0, sizeof cury_adds);
        }
    }
    (void)curz_add;
}

static dep_target make_target(to_state *s)
{
    dep_target t;
    t.cx = s->curx; t.cy = s->cury; t.cz = s->curz;
    t.fx = s->fx; t.fy = s->fy; t.fz = s->fz;
    t.scale = ldexpf(1.0f, s->fx_shift);
    t.lot = to_lot(s);
    t.fixed = s->fixed;
    return t;
}

void to_densdecomp(to_state *s, float x2, float y2, float z2, float x1, float y1, float z1, float q)
{
    dep_target t = make_target(s);
    densdecomp(s, &t, x2, y2, z2, x1, y1, z1, q);
}

void to_fixed_to_float(to_state *s)
{
    int64_t lot = to_lot(s);
    double inv = ldexp(1.0, -s->fx_shift);
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < lot; l++) {
        s->curx[l] = (float)((double)s->fx[l] * inv);
        s->cury[l] = (float)((double)s->fy[l] * inv);
        s->curz[l] = (float)((double)s->fz[l] * inv);
    }
}

/* the per-species deposit loop (:1381-1540 ions, :1715-1880 electrons):
   reconstruct the old position from the new one and the new momentum */
static void deposit_species(to_state *s, int64_t base, int64_t count, float qs)
{
    const float c = s->c;
#ifdef _OPENMP
    int nth = omp_get_max_threads();
    if (nth > 1 && count > 4096) {
        /* thread-private accumulators, summed in thread order; the serial
           build (used for parity) never takes this branch */
        int64_t lot = to_lot(s);
        float *pcur = NULL;
        int64_t *pfix = NULL;
        if (s->fixed) pfix = calloc((size_t)nth * 3 * lot, sizeof(int64_t));
        else pcur = calloc((size_t)nth * 3 * lot, sizeof(float));
#pragma omp parallel
        {
            int tid = omp_get_thread_num();
            dep_target t = make_target(s);
            if (s->fixed) {
                t.fx = pfix + (size_t)tid * 3 * lot; t.fy = t.fx + lot; t.fz = t.fy + lot;
            } else {
                t.cx = pcur + (size_t)tid * 3 * lot; t.cy = t.cx + lot; t.cz = t.cy + lot;
            }
#pragma omp for schedule(static)
            for (int64_t n = 0; n < count; n++) {
                to_particle *pp = &s->p[base + n];
                float invgam = 1.0f / sqrtf(1.0f + pp->u * pp->u + pp->v * pp->v + pp->w * pp->w);
                float x0 = pp->x - pp->u * invgam * c;
                float y0 = pp->y - pp->v * invgam * c;
                float z0 = pp->z - pp->w * invgam * c;
                float q = pp->ch * qs;
                densdecomp(s, &t, pp->x, pp->y, pp->z, x0, y0, z0, q);
            }
        }
#pragma omp parallel for schedule(static)
        for (int64_t l = 0; l < lot; l++) {
            for (int th = 0; th < nth; th++) {
                size_t b = (size_t)th * 3 * lot;
                if (s->fixed) {
                    s->fx[l] += pfix[b + l]; s->fy[l] += pfix[b + lot + l]; s->fz[l] += pfix[b + 2 * lot + l];
                } else {
                    s->curx[l] += pcur[b + l]; s->cury[l] += pcur[b + lot + l]; s->curz[l] += pcur[b + 2 * lot + l];
                }
            }
        }
        free(pcur);
        free(pfix);
        return;
    }
#endif
    dep_target t = make_target(s);
    for (int64_t n = 0; n < count; n++) {
        to_particle *pp = &s->p[base + n];
        float invgam = 1.0f / sqrtf(1.0f + pp->u * pp->u + pp->v * pp->v + pp->w * pp->w);
        float x0 = pp->x - pp->u * invgam * c;
        float y0 = pp->y - pp->v * invgam * c;
        float z0 = pp->z - pp->w * invgam * c;
        float q = pp->ch * qs;
        densdecomp(s, &t, pp->x, pp->y, pp->z, x0, y0, z0, q);
    }
}

/* boundary loop of deposit_particles (:1546-1691 ions, :1884-2026
   electrons) for one rank (sizex = sizey = 1): periodic wrap by
   +-(max-min), discard outside [x1in,x2in] on open axes, and in 3D the
   z-crossing particles routed to the z out-lists (MPI to self) */
static void boundary_species(to_state *s, int64_t base, int64_t *count, int64_t *nout,
                             to_particle **dwn, int64_t *ndwn, to_particle **up, int64_t *nup)
{
    const int nghost = s->nghost, nghostz = s->nghostz;
    const float maxx = (float)s->mx - 1.0f * (float)(nghost / 2);
    const float minx = 1.0f * (float)(nghost / 2 + 1);
    const float maxy = (float)s->my - 1.0f * (float)(nghost / 2);
    const float miny = 1.0f * (float)(nghost / 2 + 1);
    float maxz, minz;
    if (s->dims == 3) {
        maxz = (float)s->mz - 1.0f * (float)(nghostz / 2);
        minz = 1.0f * (float)(nghostz / 2 + 1);
    } else {
        minz = 1.0f * (float)(nghostz / 2 + 1);
        maxz = 1.0f * (float)(nghostz / 2 + 1) + 1.0f;
    }
    const float midx = 0.5f * (maxx - minx), midy = 0.5f * (maxy - miny), midz = 0.5f * (maxz - minz);
    int64_t n0 = *count;
    *ndwn = 0;
    *nup = 0;
    *dwn = NULL;
    *up = NULL;
    if (n0 > 0 && s->dims == 3) {
        *dwn = malloc(sizeof(to_particle) * n0);
        *up = malloc(sizeof(to_particle) * n0);
    }
    for (int64_t n = 0; n < n0; n++) {
        to_particle *pp = &s->p[base + n];
        int in = 1;
        float perx = 0.0f, pery = 0.0f, perz = 0.0f;
        if (pp->x < minx || pp->x > maxx) perx = copysignf(midx, pp->x - minx) + copysignf(midx, pp->x - maxx);
        if (pp->y < miny || pp->y > maxy) pery = copysignf(midy, pp->y - miny) + copysignf(midy, pp->y - maxy);
        if (pp->z < minz || pp->z > maxz) perz = copysignf(midz, pp->z - minz) + copysignf(midz, pp->z - maxz);
        if (s->periodic[0] == 0) {
            float xg = pp->x + (float)s->mxcum;
            in = ((double)xg > s->x1in) && ((double)xg < s->x2in);
        }
        if (s->periodic[1] == 0 && in) {
            float yg = pp->y + (float)s->mycum;
            in = ((double)yg > s->y1in) && ((double)yg < s->y2in);
        }
        if (s->dims == 3 && s->periodic[2] == 0 && in) {
            float zg = pp->z + (float)s->mzcum;
            in = ((double)zg > s->z1in) && ((double)zg < s->z2in);
        }
        if (!in) { perx = 0.0f; pery = 0.0f; perz = 0.0f; }
        pp->x = pp->x - perx;
        pp->y = pp->y - pery;
        if (s->dims == 3) {
            if (perz != 0.0f && in) { in = 0; perx = 0.0f; pery = 0.0f; }
            if (perz < 0.0f) perz = -((float)s->mz - 1.0f * (float)nghostz);
        }
        pp->z = pp->z - perz;
        if (in) continue;
        (*nout)++;
        if (s->dims == 3) {
            if (perz < 0.0f) (*dwn)[(*ndwn)++] = *pp;
            if (perz > 0.0f) (*up)[(*nup)++] = *pp;
        }
        s->pind[n] = 1;
    }
    /* compaction: swap from the end (:1694-1705, :2029-2040) */
    int64_t cnt = n0;
    for (int64_t n = 0; n < n0; n++) {
        while (s->pind[n] != 0) {
            s->p[base + n] = s->p[base + cnt - 1];
            s->pind[n] = s->pind[cnt - 1];
            s->pind[cnt - 1] = 0;
            cnt--;
        }
    }
    *count = cnt;
}

void to_deposit_particles(to_state *s)
{
    s->nionout = 0;
    s->nlecout = 0;
    if (s->ions > 0) deposit_species(s, 0, s->ions, s->qi);
    if (s->lecs > 0) deposit_species(s, s->maxhlf, s->lecs, s->qe);
    to_particle *idwn = NULL, *iup = NULL, *ldwn = NULL, *lup = NULL;
    int64_t nidwn = 0, niup = 0, nldwn = 0, nlup = 0;
    if (s->ions > 0) boundary_species(s, 0, &s->ions, &s->nionout, &idwn, &nidwn, &iup, &niup);
    if (s->lecs > 0) {
        memset(s->pind, 0, sizeof(int32_t) * s->lecs);
        boundary_species(s, s->maxhlf, &s->lecs, &s->nlecout, &ldwn, &nldwn, &lup, &nlup);
    }
    /* 3D: exchange_particles + inject_others to self append the z-crossing
       particles, first the ones that went down then up
       (code/particles.F90:1865-2125, :1368-1421; Q8 reorder) */
    for (int64_t n = 0; n < nidwn; n++) s->p[s->ions++] = idwn[n];
    for (int64_t n = 0; n < nldwn; n++) s->p[s->maxhlf + s->lecs++] = ldwn[n];
    for (int64_t n = 0; n < niup; n++) s->p[s->ions++] = iup[n];
    for (int64_t n = 0; n < nlup; n++) s->p[s->maxhlf + s->lecs++] = lup[n];
    free(idwn); free(iup); free(ldwn); free(lup);
    if (s->fixed) to_fixed_to_float(s);
}

/* ------------------------------------------------------------------------
 * Fields (code/fields.F90)
 * --------------------------------------------------------------------- */
void to_reset_currents(to_state *s)
{
    int64_t lot = to_lot(s);
    memset(s->curx, 0, sizeof(float) * lot);
    memset(s->cury, 0, sizeof(float) * lot);
    memset(s->curz, 0, sizeof(float) * lot);
    if (s->fixed) {
        memset(s->fx, 0, sizeof(int64_t) * lot);
        memset(s->fy, 0, sizeof(int64_t) * lot);
        memset(s->fz, 0, sizeof(int64_t) * lot);
    }
}

/* update ranges of advance_b_halfstep / advance_e_fullstep for one rank */
static void b_range(const to_state *s, int axis, int *a1, int *a2)
{
    int m = axis == 0 ? s->mx : axis == 1 ? s->my : s->mz;
    int ng = axis == 2 ? s->nghostz : s->nghost;
    if (axis == 2 && s->dims == 2) { *a1 = 1; *a2 = 1; return; }
    if (s->periodic[axis]) { *a1 = ng / 2 + 1; *a2 = m - (ng / 2 + 1); }
    else { *a1 = 1; *a2 = m - 1; }
}

static void e_range(const to_state *s, int axis, int *a1, int *a2)
{
    int m = axis == 0 ? s->mx : axis == 1 ? s->my : s->mz;
    int ng = axis == 2 ? s->nghostz : s->nghost;
    if (axis == 2) {
        if (s->dims == 2) { *a1 = 1; *a2 = 1; return; }
        /* Q7: fields.F90:818-819 overrides the z range unconditionally */
        *a1 = ng / 2;
        *a2 = m;
        return;
    }
    if (s->periodic[axis]) { *a1 = ng / 2 + 1; *a2 = m - (ng / 2 + 1); }
    else { *a1 = ng / 2; *a2 = m; }
}

void to_advance_b_halfstep(to_state *s)
{
    int i1, i2, j1, j2, k1, k2;
    b_range(s, 0, &i1, &i2);
    b_range(s, 1, &j1, &j2);
    b_range(s, 2, &k1, &k2);
    const float cst = s->corr * (0.5f * s->c);
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = k1; k <= k2; k++) {
        for (int j = j1; j <= j2; j++) {
            for (int i = i1; i <= i2; i++) {
                int64_t l = L3(s, i, j, k);
                if (s->dims == 3) {
                    s->bx[l] = s->bx[l] + cst * (s->ey[L3(s, i, j, k + 1)] - s->ey[l] - s->ez[L3(s, i, j + 1, k)] + s->ez[l]);
                    s->by[l] = s->by[l] + cst * (s->ez[L3(s, i + 1, j, k)] - s->ez[l] - s->ex[L3(s, i, j, k + 1)] + s->ex[l]);
                    s->bz[l] = s->bz[l] + cst * (s->ex[L3(s, i, j + 1, k)] - s->ex[l] - s->ey[L3(s, i + 1, j, k)] + s->ey[l]);
                } else {
                    s->bx[l] = s->bx[l] + cst * (-s->ez[L3(s, i, j + 1, k)] + s->ez[l]);
                    s->by[l] = s->by[l] + cst * (s->ez[L3(s, i + 1, j, k)] - s->ez[l]);
                    s->bz[l] = s->bz[l] + cst * (s->ex[L3(s, i, j + 1, k)] - s->ex[l] - s->ey[L3(s, i + 1, j, k)] + s->ey[l]);
                }
            }
        }
    }
}

void to_advance_e_fullstep(to_state *s)
{
    int i1, i2, j1, j2, k1, k2;
    e_range(s, 0, &i1, &i2);
    e_range(s, 1, &j1, &j2);
    e_range(s, 2, &k1, &k2);
    const float cst = s->corr * s->c;
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = k1; k <= k2; k++) {
        for (int j = j1; j <= j2; j++) {
            for (int i = i1; i <= i2; i++) {
                int64_t l = L3(s, i, j, k);
                if (s->dims == 3) {
                    s->ex[l] = s->ex[l] + cst * (s->by[L3(s, i, j, k - 1)] - s->by[l] - s->bz[L3(s, i, j - 1, k)] + s->bz[l]);
                    s->ey[l] = s->ey[l] + cst * (s->bz[L3(s, i - 1, j, k)] - s->bz[l] - s->bx[L3(s, i, j, k - 1)] + s->bx[l]);
                    s->ez[l] = s->ez[l] + cst * (s->bx[L3(s, i, j - 1, k)] - s->bx[l] - s->by[L3(s, i - 1, j, k)] + s->by[l]);
                } else {
                    s->ex[l] = s->ex[l] + cst * (-s->bz[L3(s, i, j - 1, k)] + s->bz[l]);
                    s->ey[l] = s->ey[l] + cst * (s->bz[L3(s, i - 1, j, k)] - s->bz[l]);
                    s->ez[l] = s->ez[l] + cst * (s->bx[L3(s, i, j - 1, k)] - s->bx[l] - s->by[L3(s, i - 1, j, k)] + s->by[l]);
                }
            }
        }
    }
}

void to_add_current(to_state *s)
{
    int64_t lot = to_lot(s);
#pragma omp parallel for schedule(static)
    for (int64_t l = 0; l < lot; l++) {
        s->ex[l] = s->ex[l] + s->curx[l];
        s->ey[l] = s->ey[l] + s->cury[l];
        s->ez[l] = s->ez[l] + s->curz[l];
    }
}

/* ------------------------------------------------------------------------
 * Ghost layers (code/fieldboundaries.F90)
 * copylayr{x,y} (:714-785) and copy_layrz1_opt (:1616-1680, MPI to self):
 * layer lt <- ls over the whole face, then nt <- ns.
 * --------------------------------------------------------------------- */
static void copy_layer(to_state *s, float *a, int axis, int t, int src)
{
    int mx = s->mx, my = s->my, mz = s->mz;
    if (axis == 0) {
        for (int k = 1; k <= mz; k++)
            for (int j = 1; j <= my; j++) a[L3(s, t, j, k)] = a[L3(s, src, j, k)];
    } else if (axis == 1) {
        for (int k = 1; k <= mz; k++)
            for (int i = 1; i <= mx; i++) a[L3(s, i, t, k)] = a[L3(s, i, src, k)];
    } else {
        for (int j = 1; j <= my; j++)
            for (int i = 1; i <= mx; i++) a[L3(s, i, j, t)] = a[L3(s, i, j, src)];
    }
}

static void copy_layrs(to_state *s, float *a, float *b, float *c, int axis, int lt, int ls, int nt, int ns)
{
    copy_layer(s, a, axis, lt, ls);
    copy_layer(s, b, axis, lt, ls);
    copy_layer(s, c, axis, lt, ls);
    copy_layer(s, a, axis, nt, ns);
    copy_layer(s, b, axis, nt, ns);
    copy_layer(s, c, axis, nt, ns);
}

static void bc_periodic(to_state *s, float *a, float *b, float *c)
{
    int ng = s->nghost;
    if (s->periodic[0])
        for (int it = 1; it <= ng / 2; it++)
            copy_layrs(s, a, b, c, 0, ng / 2 + 1 - it, s->mx - (ng / 2 + it), s->mx - (ng / 2 + 1) + it, ng / 2 + it);
    if (s->periodic[1])
        for (int it = 1; it <= ng / 2; it++)
            copy_layrs(s, a, b, c, 1, ng / 2 + 1 - it, s->my - (ng / 2 + it), s->my - (ng / 2 + 1) + it, ng / 2 + it);
    if (s->dims == 3 && s->periodic[2]) {
        int ngz = s->nghostz;
        for (int it = 1; it <= ngz / 2; it++)
            copy_layrs(s, a, b, c, 2, ngz / 2 + 1 - it, s->mz - (ngz / 2 + it), s->mz - (ngz / 2 + 1) + it, ngz / 2 + it);
    }
}

void to_bc_b1(to_state *s) { bc_periodic(s, s->bx, s->by, s->bz); }
void to_bc_e1(to_state *s) { bc_periodic(s, s->ex, s->ey, s->ez); }

/* ------------------------------------------------------------------------
 * Current ghost fold, exchange_current (code/fieldboundaries.F90:1768-2189)
 * for one rank: x then y then z. Per axis and component:
 *   cur(ng/2+1 .. ng)          += cur(m-ng/2 .. m)        (copied first)
 *   cur(m-(ng-1) .. m-(ng/2+1)) += cur(1 .. ng/2)
 * --------------------------------------------------------------------- */
static void fold_axis(to_state *s, float *a, int axis, const float *q5_src)
{
    int m = axis == 0 ? s->mx : axis == 1 ? s->my : s->mz;
    int ng = axis == 2 ? s->nghostz : s->nghost;
    int n1 = axis == 0 ? s->my : s->mx;
    int n2 = axis == 2 ? s->my : s->mz;
    int nb1 = ng / 2 + 1, nb2 = ng / 2;
    /* buffers hold the original source layers */
    float *b1 = malloc(sizeof(float) * (size_t)nb1 * n1 * n2);
    float *b2 = malloc(sizeof(float) * (size_t)nb2 * n1 * n2);
    for (int t = 0; t < nb1; t++)
        for (int q = 0; q < n2; q++)
            for (int p = 0; p < n1; p++) {
                int lay = m - ng / 2 + t;
                int64_t l;
                if (axis == 0) l = L3(s, lay, p + 1, q + 1);
                else if (axis == 1) l = L3(s, p + 1, lay, q + 1);
                else l = L3(s, p + 1, q + 1, lay);
                float v = a[l];
                /* Q5 (left-hand-side reading): the last buffer layer keeps
                   what the previous component's copy left there */
                if (q5_src && t == nb1 - 1) v = q5_src[l];
                b1[((size_t)t * n2 + q) * n1 + p] = v;
            }
    for (int t = 0; t < nb2; t++)
        for (int q = 0; q < n2; q++)
            for (int p = 0; p < n1; p++) {
                int lay = 1 + t;
                int64_t l;
                if (axis == 0) l = L3(s, lay, p + 1, q + 1);
                else if (axis == 1) l = L3(s, p + 1, lay, q + 1);
                else l = L3(s, p + 1, q + 1, lay);
                b2[((size_t)t * n2 + q) * n1 + p] = a[l];
            }
    for (int t = 0; t < nb1; t++)
        for (int q = 0; q < n2; q++)
            for (int p = 0; p < n1; p++) {
                int lay = ng / 2 + 1 + t;
                int64_t l;
                if (axis == 0) l = L3(s, lay, p + 1, q + 1);
                else if (axis == 1) l = L3(s, p + 1, lay, q + 1);
                else l = L3(s, p + 1, q + 1, lay);
                a[l] = a[l] + b1[((size_t)t * n2 + q) * n1 + p];
            }
    for (int t = 0; t < nb2; t++)
        for (int q = 0; q < n2; q++)
            for (int p = 0; p < n1; p++) {
                int lay = m - (ng - 1) + t;
                int64_t l;
                if (axis == 0) l = L3(s, lay, p + 1, q + 1);
                else if (axis == 1) l = L3(s, p + 1, lay, q + 1);
                else l = L3(s, p + 1, q + 1, lay);
                a[l] = a[l] + b2[((size_t)t * n2 + q) * n1 + p];
            }
    free(b1);
    free(b2);
}

void to_exchange_current(to_state *s)
{
    if (s->periodic[0]) {
        fold_axis(s, s->curx, 0, NULL);
        fold_axis(s, s->cury, 0, NULL);
        fold_axis(s, s->curz, 0, NULL);
    }
    if (s->periodic[1]) {
        fold_axis(s, s->curx, 1, NULL);
        fold_axis(s, s->cury, 1, (s->quirks & TO_QUIRK_Q5_LHS) ? s->curx : NULL);
        fold_axis(s, s->curz, 1, NULL);
    }
    if (s->dims == 3 && s->periodic[2]) {
        fold_axis(s, s->curx, 2, NULL);
        fold_axis(s, s->cury, 2, NULL);
        fold_axis(s, s->curz, 2, NULL);
    }
}

/* ------------------------------------------------------------------------
 * Binomial filter, apply_filter1_opt (code/filter.F90:8-221): ntimes
 * passes; each refreshes one ghost layer per side (x, y, z) and applies
 * the one-shot 9-point (2D, /16) or 27-point (3D, /64) stencil per
 * component through `temp`. The curz row range runs two rows further
 * (Q6, filter.F90:186,211).
 * --------------------------------------------------------------------- */
static void filter_component(to_state *s, float *cur, int jhi_extra)
{
    const int ng = s->nghost, ngz = s->nghostz;
    const int i1 = ng / 2 + 1, i2 = s->mx - (ng / 2 + 1);
    const int j1 = ng / 2 + 1, j2 = s->my - (ng / 2 + 1) + jhi_extra;
    int k1 = 1, k2 = 1;
    if (s->dims == 3) { k1 = ngz / 2 + 1; k2 = s->mz - (ngz / 2 + 1); }
    float *temp = s->temp;
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = k1; k <= k2; k++) {
        for (int j = j1; j <= j2; j++) {
            for (int i = i1; i <= i2; i++) {
#define C(a, b, cc) cur[L3(s, i + (a), j + (b), k + (cc))]
                float t;
                if (s->dims == 2) {
                    const float winv = 1.0f / 16.0f;
                    const float wtl = 2.0f * winv, wt = 4.0f * winv, wtr = 2.0f * winv, wtu = 2.0f * winv,
                                wtb = 2.0f * winv, wtlt = 1.0f * winv, wtrt = 1.0f * winv, wtlb = 1.0f * winv,
                                wtrb = 1.0f * winv;
                    t = wtl * C(-1, 0, 0) + wt * C(0, 0, 0) + wtr * C(1, 0, 0) + wtb * C(0, -1, 0) +
                        wtu * C(0, 1, 0) + wtlt * C(-1, 1, 0) + wtrt * C(1, 1, 0) + wtlb * C(-1, -1, 0) +
                        wtrb * C(1, -1, 0);
                } else {
                    const float winv = 1.0f / 64.0f;
                    const float wtl = 4.0f * winv, wt = 8.0f * winv, wtr = 4.0f * winv, wtu = 4.0f * winv,
                                wtb = 4.0f * winv, wtlt = 2.0f * winv, wtrt = 2.0f * winv, wtlb = 2.0f * winv,
                                wtrb = 2.0f * winv;
                    const float wtlz = 2.0f * winv, wtz = 4.0f * winv, wtrz = 2.0f * winv, wtuz = 2.0f * winv,
                                wtbz = 2.0f * winv, wtltz = 1.0f * winv, wtrtz = 1.0f * winv,
                                wtlbz = 1.0f * winv, wtrbz = 1.0f * winv;
                    t = wtl * C(-1, 0, 0) + wt * C(0, 0, 0) + wtr * C(1, 0, 0) + wtb * C(0, -1, 0) +
                        wtu * C(0, 1, 0) + wtlt * C(-1, 1, 0) + wtrt * C(1, 1, 0) + wtlb * C(-1, -1, 0) +
                        wtrb * C(1, -1, 0);
                    t = t + wtlz * C(-1, 0, -1) + wtz * C(0, 0, -1) + wtrz * C(1, 0, -1) + wtbz * C(0, -1, -1) +
                        wtuz * C(0, 1, -1) + wtltz * C(-1, 1, -1) + wtrtz * C(1, 1, -1) +
                        wtlbz * C(-1, -1, -1) + wtrbz * C(1, -1, -1) + wtlz * C(-1, 0, 1) + wtz * C(0, 0, 1) +
                        wtrz * C(1, 0, 1) + wtbz * C(0, -1, 1) + wtuz * C(0, 1, 1) + wtltz * C(-1, 1, 1) +
                        wtrtz * C(1, 1, 1) + wtlbz * C(-1, -1, 1) + wtrbz * C(1, -1, 1);
                }
#undef C
                temp[L3(s, i, j, k)] = t;
            }
        }
    }
#pragma omp parallel for schedule(static) collapse(2)
    for (int k = k1; k <= k2; k++)
        for (int j = j1; j <= j2; j++)
            for (int i = i1; i <= i2; i++) cur[L3(s, i, j, k)] = temp[L3(s, i, j, k)];
}

void to_apply_filter1_opt(to_state *s)
{
    const int ng = s->nghost, ngz = s->nghostz;
    for (int n = 1; n <= s->ntimes; n++) {
        /* one ghost layer per side; copy_layr{x,y,z}1_opt with
           lt=ng/2, ls=m-(ng/2+1), nt=m-ng/2, ns=ng/2+1 */
        if (s->periodic[0])
            copy_layrs(s, s->curx, s->cury, s->curz, 0, ng / 2, s->mx - (ng / 2 + 1), s->mx - ng / 2, ng / 2 + 1);
        if (s->periodic[1])
            copy_layrs(s, s->curx, s->cury, s->curz, 1, ng / 2, s->my - (ng / 2 + 1), s->my - ng / 2, ng / 2 + 1);
        if (s->dims == 3 && s->periodic[2])
            copy_layrs(s, s->curx, s->cury, s->curz, 2, ngz / 2, s->mz - (ngz / 2 + 1), s->mz - ngz / 2, ngz / 2 + 1);
        filter_component(s, s->curx, 0);
        filter_component(s, s->cury, 0);
        filter_component(s, s->curz, 2);
    }
}

/* ------------------------------------------------------------------------
 * Reorder (code/particles.F90:394-497): every 10 laps except the lap right
 * after the previous reorder, stable counting sort by
 * celli = int(x) + int(y)*iy + int(z)*iz (iz = 0 in 2D).
 * --------------------------------------------------------------------- */
static void reorder_range(to_state *s, int64_t base, int64_t count)
{
    const int64_t iy = s->mx, iz = s->dims == 3 ? (int64_t)s->mx * s->my : 0;
    const int64_t lot = to_lot(s);
    memset(s->pall, 0, sizeof(int32_t) * (lot + 1));
    for (int64_t n = 0; n < count; n++) {
        const to_particle *pp = &s->p[base + n];
        int64_t celli = (int64_t)(int)pp->x + (int64_t)(int)pp->y * iy + (int64_t)(int)pp->z * iz;
        if (celli < 1 || celli > lot) celli = lot; /* out of range: keep, sort last */
        s->pall[celli]++;
    }
    int64_t kacc = 1;
    for (int64_t i = 1; i <= lot; i++) {
        int64_t j = s->pall[i];
        s->pall[i] = (int32_t)kacc;
        kacc += j;
    }
    for (int64_t n = 0; n < count; n++) {
        const to_particle *pp = &s->p[base + n];
        int64_t celli = (int64_t)(int)pp->x + (int64_t)(int)pp->y * iy + (int64_t)(int)pp->z * iz;
        if (celli < 1 || celli > lot) celli = lot;
        int64_t j = s->pall[celli];
        s->pall[celli]++;
        s->tempp[j - 1] = *pp;
    }
    memcpy(&s->p[base], s->tempp, sizeof(to_particle) * count);
}

void to_reorder_particles_(to_state *s)
{
    reorder_range(s, 0, s->ions);
    reorder_range(s, s->maxhlf, s->lecs);
}

void to_reorder_particles(to_state *s)
{
    if (s->lap == s->lapreorder + 1) return;
    if (s->lap % 10 != 0) return;
    to_reorder_particles_(s);
    s->lapreorder = s->lap;
}

/* ------------------------------------------------------------------------
 * One lap (code/tristanmainloop.F90:107-344) for periodic boxes without
 * radiation boundaries, injection or user particle BCs.
 * --------------------------------------------------------------------- */
void to_step(to_state *s)
{
    to_bc_b1(s);
    to_bc_e1(s);
    to_advance_b_halfstep(s);
    to_bc_b1(s);
    to_move_particles(s);
    to_advance_b_halfstep(s);
    to_bc_b1(s);
    to_bc_b1(s); /* bc_b2 without radiation boundaries */
    to_advance_e_fullstep(s);
    to_bc_e1(s); /* bc_e2 */
    to_reset_currents(s);
    to_bc_e1(s);
    to_bc_b1(s);
    to_deposit_particles(s);
    to_exchange_current(s);
    to_apply_filter1_opt(s);
    to_add_current(s);
    to_reorder_particles(s);
    s->lap++;
}

/* ------------------------------------------------------------------------
 * FP64 diagnostics. rho is deposited on the interior nodes with the same
 * B-spline (the Esirkepov deposit conserves exactly this rho), wrapped
 * periodically, then filtered ntimes with the current filter's stencil.
 * div E uses backward differences at nodes (E is staggered forward).
 * --------------------------------------------------------------------- */
static inline int wrapi(int i, int lo, int n) { return lo + ((i - lo) % n + n) % n; }

void to_charge_density(const to_state *s, double *rho)
{
    const int ng = s->nghost, ngz = s->nghostz;
    const int lo = ng / 2 + 1, nx = s->mx - ng, ny = s->my - ng;
    const int loz = s->dims == 3 ? ngz / 2 + 1 : 1, nz = s->dims == 3 ? s->mz - ngz : 1;
    const int64_t lot = to_lot(s);
    memset(rho, 0, sizeof(double) * lot);
    for (int sp = 0; sp < 2; sp++) {
        int64_t base = sp == 0 ? 0 : s->maxhlf;
        int64_t cnt = sp == 0 ? s->ions : s->lecs;
        double qs = sp == 0 ? s->qi : s->qe;
        for (int64_t n = 0; n < cnt; n++) {
            const to_particle *pp = &s->p[base + n];
            float Sx[8] = {0}, Sy[8] = {0}, Sz[8] = {0};
            int xm, xM, ym, yM, zm = 3, zM = 3;
            int i = (int)truncf(pp->x), j = (int)truncf(pp->y), k = (int)truncf(pp->z);
            shape(s->order, pp->x - truncf(pp->x), Sx, 0, &xm, &xM);
            shape(s->order, pp->y - truncf(pp->y), Sy, 0, &ym, &yM);
            if (s->dims == 3) shape(s->order, pp->z - truncf(pp->z), Sz, 0, &zm, &zM);
            else { Sz[3] = 1.0f; k = 1; }
            double q = (double)pp->ch * qs;
            for (int c = zm; c <= zM; c++)
                for (int b = ym; b <= yM; b++)
                    for (int a = xm; a <= xM; a++) {
                        int ii = wrapi(i - 3 + a, lo, nx), jj = wrapi(j - 3 + b, lo, ny);
                        int kk = s->dims == 3 ? wrapi(k - 3 + c, loz, nz) : 1;
                        rho[L3(s, ii, jj, kk)] += q * (double)Sx[a] * (double)Sy[b] * (double)Sz[c];
                    }
        }
    }
    /* filter ntimes on the periodic interior */
    double *tmp = malloc(sizeof(double) * lot);
    for (int pass = 0; pass < s->ntimes; pass++) {
        memcpy(tmp, rho, sizeof(double) * lot);
        for (int k = loz; k < loz + nz; k++)
            for (int j = lo; j < lo + ny; j++)
                for (int i = lo; i < lo + nx; i++) {
                    double acc = 0.0;
                    for (int dc = (s->dims == 3 ? -1 : 0); dc <= (s->dims == 3 ? 1 : 0); dc++)
                        for (int db = -1; db <= 1; db++)
                            for (int da = -1; da <= 1; da++) {
                                double w = (da == 0 ? 2.0 : 1.0) * (db == 0 ? 2.0 : 1.0) *
                                           (s->dims == 3 ? (dc == 0 ? 2.0 : 1.0) : 1.0);
                                int kk = s->dims == 3 ? wrapi(k + dc, loz, nz) : 1;
                                acc += w * tmp[L3(s, wrapi(i + da, lo, nx), wrapi(j + db, lo, ny), kk)];
                            }
                    rho[L3(s, i, j, k)] = acc / (s->dims == 3 ? 64.0 : 16.0);
                }
    }
    free(tmp);
}

void to_diagnostics(const to_state *s, to_diag *out)
{
    const int ng = s->nghost, ngz = s->nghostz;
    const int lo = ng / 2 + 1, nx = s->mx - ng, ny = s->my - ng;
    const int loz = s->dims == 3 ? ngz / 2 + 1 : 1, nz = s->dims == 3 ? s->mz - ngz : 1;
    const int64_t lot = to_lot(s);
    double *rho = malloc(sizeof(double) * lot);
    to_charge_density(s, rho);
    memset(out, 0, sizeof *out);
    double r2 = 0.0, d2 = 0.0;
    for (int k = loz; k < loz + nz; k++)
        for (int j = lo; j < lo + ny; j++)
            for (int i = lo; i < lo + nx; i++) {
                int64_t l = L3(s, i, j, k);
                double div = (double)s->ex[l] - (double)s->ex[L3(s, wrapi(i - 1, lo, nx), j, k)] +
                             (double)s->ey[l] - (double)s->ey[L3(s, i, wrapi(j - 1, lo, ny), k)];
                if (s->dims == 3) div += (double)s->ez[l] - (double)s->ez[L3(s, i, j, wrapi(k - 1, loz, nz))];
                double r = div - rho[l];
                d2 += r * r;
                r2 += rho[l] * rho[l];
                out->charge_total += rho[l];
                double ex = s->ex[l], ey = s->ey[l], ez = s->ez[l], bx = s->bx[l], by = s->by[l], bz = s->bz[l];
                out->e_field += 0.5 * (ex * ex + ey * ey + ez * ez);
                out->e_mag += 0.5 * (bx * bx + by * by + bz * bz);
                out->p_field[0] += ey * bz - ez * by;
                out->p_field[1] += ez * bx - ex * bz;
                out->p_field[2] += ex * by - ey * bx;
            }
    out->gauss_abs = sqrt(d2);
    out->rho_norm = sqrt(r2);
    out->gauss_residual = r2 > 0.0 ? sqrt(d2 / r2) : sqrt(d2);
    for (int sp = 0; sp < 2; sp++) {
        int64_t base = sp == 0 ? 0 : s->maxhlf;
        int64_t cnt = sp == 0 ? s->ions : s->lecs;
        double m = sp == 0 ? fabs((double)s->qi / (double)s->qmi) : fabs((double)s->qe / (double)s->qme);
        double ek = 0.0;
        for (int64_t n = 0; n < cnt; n++) {
            const to_particle *pp = &s->p[base + n];
            double u = pp->u, v = pp->v, w = pp->w, ch = pp->ch;
            double gam = sqrt(1.0 + u * u + v * v + w * w);
            ek += (gam - 1.0) * m * ch;
            out->p_part[0] += m * ch * u;
            out->p_part[1] += m * ch * v;
            out->p_part[2] += m * ch * w;
        }
        if (sp == 0) out->e_kin_ions = ek;
        else out->e_kin_lecs = ek;
    }
    free(rho);
}

/* ------------------------------------------------------------------------
 * Collisionless-shock setup, 2D (user_pu/user_shock_pu.F90 with wall = 1,
 * rightclean = 0, rightwall = 0, wallgam from the input).
 * --------------------------------------------------------------------- */

/* Park-Miller minimal standard generator, code/aux.F90:82-99: the seed is
   an integer held in a double, SEED = DMOD(16807*SEED, 2^31-1) (exact in
   double), returned as SEED/2^31 rounded to single */
float to_random(double *dseed)
{
    double seed;
    const int64_t si = (int64_t)*dseed;
    if ((double)si == *dseed && si >= 0 && si < 2147483647LL)
        seed = (double)((16807LL * si) % 2147483647LL); /* the same exact integer, without fmod */
    else
        seed = fmod(16807.0 * *dseed, 2147483647.0);
    *dseed = seed;
    return (float)(seed / 2147483648.0);
}

/* code/aux.F90:110-134 */
float to_poisson(float numps, double *dseed)
{
    double Lps = exp(-(double)numps);
    float kps = 0.0f;
    double pps = 1.0;
    while (pps >= Lps) {
        kps = kps + 1.0f;
        float ups = to_random(dseed);
        pps = pps * (double)ups;
    }
    return kps - 1.0f;
}

/* sin and cos of a float: reduction by pi/2 in double (pi/2 split into a
   33-bit head and a tail, so k * head is exact), Taylor series to degree
   17 on |r| <= pi/4, one rounding to single at the end */
static double sin_taylor(double r)
{
    const double r2 = r * r;
    double t = 1.0 / 355687428096000.0;               /* 1/17! */
    t = 1.0 / 1307674368000.0 - r2 * t;               /* 1/15! */
    t = 1.0 / 6227020800.0 - r2 * t;                  /* 1/13! */
    t = 1.0 / 39916800.0 - r2 * t;                    /* 1/11! */
    t = 1.0 / 362880.0 - r2 * t;                      /* 1/9!  */
    t = 1.0 / 5040.0 - r2 * t;                        /* 1/7!  */
    t = 1.0 / 120.0 - r2 * t;                         /* 1/5!  */
    t = 1.0 / 6.0 - r2 * t;                           /* 1/3!  */
    return r - r * r2 * t;
}

static double cos_taylor(double r)
{
    const double r2 = r * r;
    double t = 1.0 / 20922789888000.0;                /* 1/16! */
    t = 1.0 / 87178291200.0 - r2 * t;                 /* 1/14! */
    t = 1.0 / 479001600.0 - r2 * t;                   /* 1/12! */
    t = 1.0 / 3628800.0 - r2 * t;                     /* 1/10! */
    t = 1.0 / 40320.0 - r2 * t;                       /* 1/8!  */
    t = 1.0 / 720.0 - r2 * t;                         /* 1/6!  */
    t = 1.0 / 24.0 - r2 * t;                          /* 1/4!  */
    t = 0.5 - r2 * t;                                 /* 1/2!  */
    return 1.0 - r2 * t;
}

void to_sincosf(float x, float *sn, float *cs)
{
    const double PIO2_HI = 0x1.921fb544p+0, PIO2_LO = 0x1.0b4611a626331p-34, TWO_OVER_PI = 0x1.45f306dc9c883p-1;
    const double xd = (double)x;
    const double k = nearbyint(xd * TWO_OVER_PI);
    const double r = (xd - k * PIO2_HI) - k * PIO2_LO;
    const double s = sin_taylor(r), c = cos_taylor(r);
    const long q = ((long)k) & 3;
    double so, co;
    if (q == 0) { so = s; co = c; }
    else if (q == 1) { so = c; co = -s; }
    else if (q == 2) { so = -s; co = -c; }
    else { so = -c; co = s; }
    *sn = (float)so;
    *cs = (float)co;
}

/* code/particles.F90:2126-2163 */
void to_init_maxw_table(float delgam, int dims, float pcosthmult, float *gt, float *pt)
{
    float maxg = delgam * 20.0f + 1.0f;
    float func[TO_PDF_SZ];
    for (int i = 1; i <= TO_PDF_SZ; i++)
        gt[i - 1] = (maxg - 1.0f) / (float)(TO_PDF_SZ - 1) * (float)(i - 1);
    for (int i = 0; i < TO_PDF_SZ; i++) {
        const float g = gt[i];
        if (dims == 3 || pcosthmult == 1.0f)
            func[i] = (g + 1.0f) * sqrtf(g * (g + 2.0f)) * expf(-g / delgam);
        else
            func[i] = (g + 1.0f) * expf(-g / delgam);
    }
    pt[0] = 0.0f;
    float sum = 0.0f;
    for (int i = 1; i <= TO_PDF_SZ; i++) {
        sum = sum + func[i - 1];
        pt[i] = sum;
    }
    /* the whole array divided by its element pdf_sz (1-based), read before
       the assignment */
    const float norm = pt[TO_PDF_SZ - 1];
    for (int i = 0; i <= TO_PDF_SZ; i++) pt[i] = pt[i] / norm;
}

/* code/particles.F90:2176-2273, 2D build (pcosth drawn once more when
   sigma != 0); pi is the double of the single literal 3.1415927 */
void to_maxwell_dist(float gamma0, float cd, double *dseed, float *u, float *v, float *w, const float *gt,
                     const float *pt, float pcosthmult, int sigma_nonzero)
{
    const double pi = (double)3.1415927f;
    const float gamma0mag = fabsf(gamma0);
    const float gm = fmaxf(fabsf(gamma0), 1.0f);
    const float beta_drift = copysignf(sqrtf(1.0f - 1.0f / (gm * gm)), gamma0);
    float rannum = to_random(dseed);
    if (rannum == 1.0f) rannum = to_random(dseed);
    /* The reference scans i = 1, 2, ... for the first interval with
       pdf(i) <= rannum < pdf(i+1), stopping at i = pdf_sz. The table is
       non-decreasing from pdf(1) = 0 <= rannum, so that interval is the one
       whose upper end is the first entry above rannum: a binary search for
       it gives the same i. */
    int lo = 1, hi = TO_PDF_SZ; /* first 1-based i in [1, pdf_sz) with pt[i] > rannum, else pdf_sz */
    while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (pt[mid] > rannum) hi = mid;
        else lo = mid + 1;
    }
    float gam;
    if (lo >= TO_PDF_SZ) {
        gam = gt[TO_PDF_SZ - 1];
    } else {
        const int i = lo;
        gam = gt[i - 1] + (gt[i] - gt[i - 1]) / (pt[i] - pt[i - 1]) * (rannum - pt[i - 1]);
    }
    float pcosth = (2.0f * to_random(dseed) - 1.0f) * pcosthmult;
    if (sigma_nonzero) pcosth = 2.0f * to_random(dseed) - 1.0f;
    const float pphi = (float)((double)(to_random(dseed) * 2.0f) * pi);
    const float psinth = sqrtf(1.0f - pcosth * pcosth);
    const float v0t = cd * sqrtf(gam * (gam + 2.0f)) / (1.0f + gam);
    float sphi, cphi;
    to_sincosf(pphi, &sphi, &cphi);
    const float ut1 = v0t * psinth * cphi;
    const float vt1 = v0t * psinth * sphi;
    const float wt1 = v0t * pcosth;
    float ptx = (1.0f + gam) * ut1;
    const float pty = (1.0f + gam) * vt1;
    const float ptz = (1.0f + gam) * wt1;
    const float X7 = to_random(dseed);
    if (-beta_drift * ut1 / cd > X7) ptx = -ptx;
    const float px1 = (ptx + cd * beta_drift * (gam + 1.0f)) * gamma0mag;
    *u = px1 / cd;
    *v = pty / cd;
    *w = ptz / cd;
}

/* code/particles.F90:2549-2938, drift along x, one electron per ion,
   no density profile: ions and electrons appended pairwise at one point */
static void inject_region(to_state *s, to_shock *k, float x1, float x2, float y1, float y2, float z1, float z2,
                          float ppc, float weight)
{
    const int ng = s->nghost, ngz = s->nghostz;
    const float gdi = k->gamma_drift;
    const float gamma_drift = fabsf(gdi) < 1.0f ? copysignf(sqrtf(1.0f / (1.0f - gdi * gdi)), gdi) : gdi;
    const int64_t iglob_min = (ng / 2 + 1) + s->mxcum, iglob_max = (s->mx - ng / 2) + s->mxcum;
    float minx = (float)(ng / 2 + 1), maxx = (float)(ng / 2 + 1);
    if (x1 < (float)iglob_min) minx = (float)(ng / 2 + 1);
    if (x2 < (float)iglob_min) maxx = (float)(ng / 2 + 1);
    if (x1 >= (float)iglob_max) minx = (float)(s->mx - ng / 2);
    if (x2 >= (float)iglob_max) maxx = (float)(s->mx - ng / 2);
    if (x1 >= (float)iglob_min && x1 < (float)iglob_max) minx = x1 - 1.0f * (float)s->mxcum;
    if (x2 >= (float)iglob_min && x2 < (float)iglob_max) maxx = x2 - 1.0f * (float)s->mxcum;
    const float delta_x = maxx - minx;
    const int64_t jglob_min = (ng / 2 + 1) + s->mycum, jglob_max = (s->my - ng / 2) + s->mycum;
    float miny = (float)(ng / 2 + 1), maxy = (float)(ng / 2 + 1);
    if (y1 < (float)jglob_min) miny = (float)(ng / 2 + 1);
    if (y2 < (float)jglob_min) maxy = (float)(ng / 2 + 1);
    if (y1 >= (float)jglob_max) miny = (float)(s->my - ng / 2);
    if (y2 >= (float)jglob_max) maxy = (float)(s->my - ng / 2);
    if (y1 >= (float)jglob_min && y1 < (float)jglob_max) miny = y1 - (float)s->mycum;
    if (y2 >= (float)jglob_min && y2 < (float)jglob_max) maxy = y2 - (float)s->mycum;
    float delta_y = maxy - miny;
    if (maxy == 0.0f || miny == 0.0f) {
        delta_y = 0.0f;
        maxy = 0.0f;
        miny = 0.0f;
    }
    float minz, maxz, delta_z;
    if (s->dims == 2) {
        maxz = 1.0f * (float)(ngz / 2 + 1) + 1.0f;
        minz = 1.0f * (float)(ngz / 2 + 1);
        delta_z = maxz - minz;
    } else {
        /* code/particles.F90:2695-2728: z as y, on this rank's slab */
        const int64_t kglob_min = (ngz / 2 + 1) + s->mzcum, kglob_max = (s->mz - ngz / 2) + s->mzcum;
        minz = 1.0f * (float)(ngz / 2 + 1);
        maxz = 1.0f * (float)(ngz / 2 + 1);
        if (z1 < (float)kglob_min) minz = 1.0f * (float)(ngz / 2 + 1);
        if (z2 < (float)kglob_min) maxz = 1.0f * (float)(ngz / 2 + 1);
        if (z1 >= (float)kglob_max) minz = (float)s->mz - 1.0f * (float)(ngz / 2);
        if (z2 >= (float)kglob_max) maxz = (float)s->mz - 1.0f * (float)(ngz / 2);
        if (z1 >= (float)kglob_min && z1 < (float)kglob_max) minz = z1 - (float)s->mzcum;
        if (z2 >= (float)kglob_min && z2 < (float)kglob_max) maxz = z2 - (float)s->mzcum;
        delta_z = maxz - minz;
        if (maxz == 0.0f || minz == 0.0f) {
            delta_z = 0.0f;
            maxz = 0.0f;
            minz = 0.0f;
        }
    }
    float numps = (0.5f * ppc) * delta_z * delta_y * delta_x;
    if (numps < 10.0f) numps = numps != 0.0f ? to_poisson(numps, &k->dseed) : 0.0f;
    else numps = (float)(int32_t)ceilf(numps);
    const int64_t n = (int64_t)(int32_t)numps;
    if (s->ions + n > s->maxhlf || s->lecs + n > s->maxhlf) {
        k->injected = -1; /* check_overflow_num would stop the run */
        return;
    }
    for (int64_t m = 0; m < n; m++) {
        to_particle *pi = &s->p[s->ions++];
        pi->x = minx + delta_x * to_random(&k->dseed);
        pi->y = miny + delta_y * to_random(&k->dseed);
        pi->z = minz + delta_z * to_random(&k->dseed);
        to_maxwell_dist(gamma_drift, s->c, &k->dseed, &pi->u, &pi->v, &pi->w, k->gamma_table_i, k->pdf_table_i,
                        k->pcosthmult, k->sigma_nonzero);
        pi->ch = weight;
        pi->ind = ++k->totalpartnum;
        pi->proc = 0;
        pi->splitlev = 1;
        to_particle *pe = &s->p[s->maxhlf + s->lecs++];
        pe->x = pi->x;
        pe->y = pi->y;
        pe->z = pi->z;
        pe->ch = weight / 1.0f;
        to_maxwell_dist(gamma_drift, s->c, &k->dseed, &pe->u, &pe->v, &pe->w, k->gamma_table_e, k->pdf_table_e,
                        k->pcosthmult, k->sigma_nonzero);
        pe->ind = ++k->totalpartnum;
        pe->proc = 0;
        pe->splitlev = 1;
    }
    k->injected += n;
}

void to_inject_plasma_region(to_state *s, to_shock *k, float x1, float x2, float y1, float y2, float ppc,
                             float weight)
{
    inject_region(s, k, x1, x2, y1, y2, 0.0f, 0.0f, ppc, weight);
}

/* the same with the z range of a 3D build (z1, z2 ignored in 2D) */
void to_inject_plasma_region3(to_state *s, to_shock *k, float x1, float x2, float y1, float y2, float z1, float z2,
                              float ppc, float weight)
{
    inject_region(s, k, x1, x2, y1, y2, z1, z2, ppc, weight);
}

/* inject_from_wall (code/particles.F90:2439-2538) for a wall normal to x at
   x1, then the injector's bookkeeping of inject_particles_user
   (user_shock_pu.F90:364-395 with rightclean = 0, rightwall = 0) */
void to_inject_particles_user(to_state *s, to_shock *k)
{
    k->injected = 0;
    if (!k->inject) return;
    const float c = s->c;
    k->xinject2 = k->xinject2 + (double)(c * k->betainj);
    if (k->xinject2 > k->xinj_max) {
        k->xinject2 = k->xinj_max;
        k->betainj = 0.0f;
    }
    const float wall_speed = k->betainj;
    const float x1 = (float)k->xinject2;
    const float beta_wall = fabsf(wall_speed) >= 1.0f
                                ? copysignf(sqrtf(1.0f - 1.0f / (wall_speed * wall_speed)), wall_speed)
                                : wall_speed;
    const float gd = k->gamma_drift;
    const float beta_inj = fabsf(gd) >= 1.0f ? copysignf(sqrtf(1.0f - 1.0f / (gd * gd)), gd) : gd;
    float x1new = x1, x2new = x1 + (beta_inj - beta_wall) * c;
    if (x2new < x1new) {
        const float xt = x1new;
        x1new = x2new;
        x2new = xt;
    }
    to_inject_plasma_region(s, k, x1new, x2new, k->y1, k->y2, k->ppc0, k->weight);
    s->x1in = 3.0;
    s->x2in = k->xinject2;
}

/* zigzag (code/particles.F90:550-669), 2D: first-order deposit of the
   segment (x1,y1) -> (x2,y2) through the relay point */
static void zigzag(to_state *s, const dep_target *t, float x2, float y2, float z2, float x1, float y1, float z1,
                   float q)
{
    const int64_t iy = s->mx;
    const int i1 = (int)truncf(x1), i2 = (int)truncf(x2);
    const int j1 = (int)truncf(y1), j2 = (int)truncf(y2);
    int k1 = (int)truncf(z1), k2 = (int)truncf(z2);
    const float xr = fminf((float)((i1 < i2 ? i1 : i2) + 1), fmaxf((float)(i1 > i2 ? i1 : i2), 0.5f * (x1 + x2)));
    const float yr = fminf((float)((j1 < j2 ? j1 : j2) + 1), fmaxf((float)(j1 > j2 ? j1 : j2), 0.5f * (y1 + y2)));
    const float zr = fminf((float)((k1 < k2 ? k1 : k2) + 1), fmaxf((float)(k1 > k2 ? k1 : k2), 0.5f * (z1 + z2)));
    k1 = 1;
    k2 = 1;
    const float Fx1 = -q * (xr - x1), Fy1 = -q * (yr - y1), Fz1 = -q * (zr - z1);
    const float Wx1 = 0.5f * (x1 + xr) - (float)i1, Wy1 = 0.5f * (y1 + yr) - (float)j1;
    const float Wx2 = 0.5f * (x2 + xr) - (float)i2, Wy2 = 0.5f * (y2 + yr) - (float)j2;
    const float Fx2 = -q * (x2 - xr), Fy2 = -q * (y2 - yr), Fz2 = -q * (z2 - zr);
    const float Wz1 = 0.0f, Wz2 = 0.0f;
#define ZL(i, j) ((int64_t)((i) - 1) + iy * (int64_t)((j) - 1))
    (void)k1; (void)k2;
    dep_add(t, 0, ZL(i1, j1), Fx1 * (1.0f - Wy1) * (1.0f - Wz1));
    dep_add(t, 0, ZL(i1, j1 + 1), Fx1 * Wy1 * (1.0f - Wz1));
    dep_add(t, 0, ZL(i2, j2), Fx2 * (1.0f - Wy2) * (1.0f - Wz2));
    dep_add(t, 0, ZL(i2, j2 + 1), Fx2 * Wy2 * (1.0f - Wz2));
    dep_add(t, 1, ZL(i1, j1), Fy1 * (1.0f - Wx1) * (1.0f - Wz1));
    dep_add(t, 1, ZL(i1 + 1, j1), Fy1 * Wx1 * (1.0f - Wz1));
    dep_add(t, 1, ZL(i2, j2), Fy2 * (1.0f - Wx2) * (1.0f - Wz2));
    dep_add(t, 1, ZL(i2 + 1, j2), Fy2 * Wx2 * (1.0f - Wz2));
    dep_add(t, 2, ZL(i1, j1), Fz1 * (1.0f - Wx1) * (1.0f - Wy1));
    dep_add(t, 2, ZL(i1 + 1, j1), Fz1 * Wx1 * (1.0f - Wy1));
    dep_add(t, 2, ZL(i1, j1 + 1), Fz1 * (1.0f - Wx1) * Wy1);
    dep_add(t, 2, ZL(i1 + 1, j1 + 1), Fz1 * Wx1 * Wy1);
    dep_add(t, 2, ZL(i2, j2), Fz2 * (1.0f - Wx2) * (1.0f - Wy2));
    dep_add(t, 2, ZL(i2 + 1, j2), Fz2 * Wx2 * (1.0f - Wy2));
    dep_add(t, 2, ZL(i2, j2 + 1), Fz2 * (1.0f - Wx2) * Wy2);
    dep_add(t, 2, ZL(i2 + 1, j2 + 1), Fz2 * Wx2 * Wy2);
#undef ZL
}

/* left reflecting wall, user_shock_pu.F90:514-611: a particle found behind
   the wall is traced back to the crossing, deposits its path up to the
   wall (zigzag), is reflected with the wall's kick and moved forward for
   the rest of the step, and the behind-the-wall path that the deposit will
   add is cancelled (zigzag with -q); a particle that cannot have crossed
   this step is removed (the last particle of the species takes its slot) */
void to_particle_bc_user(to_state *s, to_shock *k)
{
    if (!k->wall) return;
    const float c = s->c;
    const float gammawall = k->gammawall, betawall = k->betawall;
    k->walloc = k->walloc + (double)(betawall * c);
    dep_target t = make_target(s);
    for (int iter = 0; iter < 2; iter++) {
        const int64_t base = iter == 0 ? 0 : s->maxhlf;
        int64_t *cnt = iter == 0 ? &s->ions : &s->lecs;
        const float q0 = iter == 0 ? s->qi : s->qe;
        int64_t i1 = *cnt;
        int64_t n1 = 0;
        while (n1 < i1) {
            to_particle *p = &s->p[base + n1];
            if ((double)(p->x + (float)s->mxcum) < k->walloc) {
                float gamma = sqrtf(1.0f + (p->u * p->u + p->v * p->v + p->w * p->w));
                const float x0 = p->x - p->u / gamma * c;
                const float y0 = p->y, z0 = p->z;
                const double walloc0 = k->walloc - (double)(betawall * c) - (double)s->mxcum;
                float tfrac = (float)fabs(((double)x0 - walloc0) / (double)(betawall * c - p->u / gamma * c));
                if (tfrac < 1.0f) {
                    const float xcolis = x0 + p->u / gamma * c * tfrac;
                    const float ycolis = y0, zcolis = z0;
                    float q = p->ch * q0;
                    zigzag(s, &t, xcolis, ycolis, zcolis, x0, y0, z0, q);
                    p->u = gammawall * gammawall * gamma * (2.0f * betawall - p->u / gamma * (1.0f + betawall * betawall));
                    gamma = sqrtf(1.0f + (p->u * p->u + p->v * p->v + p->w * p->w));
                    tfrac = fminf(fabsf((p->x - xcolis) / fmaxf(fabsf(p->x - x0), 1e-9f)), 1.0f);
                    p->x = xcolis + p->u / gamma * c * tfrac;
                    p->y = ycolis;
                    p->z = zcolis;
                    q = -q;
                    zigzag(s, &t, xcolis, ycolis, zcolis, p->x - p->u / gamma * c, p->y - p->v / gamma * c,
                           p->z - p->w / gamma * c, q);
                } else {
                    s->p[base + n1] = s->p[base + i1 - 1];
                    i1--;
                    continue;
                }
            }
            n1++;
        }
        *cnt = i1;
    }
}

/* user_shock_pu.F90:460-488 (rightclean = 0): conductor behind the wall,
   upstream fields at the right edge */
void to_field_bc_user(to_state *s, const to_shock *k)
{
    const int64_t iy = s->mx, iz = (int64_t)s->mx * s->my;
    for (int kk = 1; kk <= s->mz; kk++)
        for (int j = 1; j <= s->my; j++) {
            const int64_t row = iy * (j - 1) + iz * (kk - 1);
            if (k->cond_i1 != k->cond_i2)
                for (int i = k->cond_i1; i <= k->cond_i2; i++) {
                    s->ey[row + i - 1] = 0.0f;
                    s->ez[row + i - 1] = 0.0f;
                }
            if (k->edge_i1 != k->edge_i2)
                for (int i = k->edge_i1; i <= k->edge_i2; i++) {
                    s->bx[row + i - 1] = k->edge[3];
                    s->by[row + i - 1] = k->edge[4];
                    s->bz[row + i - 1] = k->edge[5];
                    s->ex[row + i - 1] = k->edge[0];
                    s->ey[row + i - 1] = k->edge[1];
                    s->ez[row + i - 1] = k->edge[2];
                }
        }
}

/* code/tristanmainloop.F90:117-303 with the user hooks (no radiation
   boundaries: bc_b2 / bc_e2 are bc_b1 / bc_e1) */
void to_step_shock(to_state *s, to_shock *k)
{
    to_bc_b1(s);
    to_bc_e1(s);
    to_advance_b_halfstep(s);
    to_bc_b1(s);
    to_move_particles(s);
    to_advance_b_halfstep(s);
    to_bc_b1(s);
    to_bc_b1(s);
    to_field_bc_user(s, k);
    to_advance_e_fullstep(s);
    to_field_bc_user(s, k);
    to_bc_e1(s);
    to_field_bc_user(s, k);
    to_reset_currents(s);
    to_particle_bc_user(s, k);
    to_bc_e1(s);
    to_bc_b1(s);
    to_deposit_particles(s);
    to_exchange_current(s);
    to_apply_filter1_opt(s);
    to_add_current(s);
    to_field_bc_user(s, k);
    to_inject_particles_user(s, k);
    to_reorder_particles(s);
    s->lap++;
}

/* ------------------------------------------------------------------------
 * Grid moments of the particles (meanq_fld_cur, code/output.F90:5222-5482):
 * every particle adds its quantity (and its weight) to the cells of a
 * (2 idx + 1) x (2 idy + 1) [x (2 idz + 1)] box around its cell, the ghost
 * layers are folded (exchange_current), each cell is divided by its box
 * size, and for the velocity-like moments by the summed weight.
 * --------------------------------------------------------------------- */
void to_meanq(to_state *s, int kind, int idx, int idy, int idz, float *num, float *den)
{
    const int64_t lot = to_lot(s);
    float *cx = s->curx, *cy = s->cury, *cz = s->curz;
    /* the reference computes into the current arrays: keep them */
    float *keep = malloc(sizeof(float) * 3 * lot);
    memcpy(keep, cx, sizeof(float) * lot);
    memcpy(keep + lot, cy, sizeof(float) * lot);
    memcpy(keep + 2 * lot, cz, sizeof(float) * lot);
    memset(cx, 0, sizeof(float) * lot);
    memset(cy, 0, sizeof(float) * lot);
    memset(cz, 0, sizeof(float) * lot);
    const int64_t iy = s->mx, iz = (int64_t)s->mx * s->my;
    for (int sp = 0; sp < 2; sp++) {
        const int64_t base = sp == 0 ? 0 : s->maxhlf, cnt = sp == 0 ? s->ions : s->lecs;
        for (int64_t n = 0; n < cnt; n++) {
            const to_particle *p = &s->p[base + n];
            const float gamprt = 1.0f / sqrtf(1.0f + p->u * p->u + p->v * p->v + p->w * p->w);
            float ax = 0.0f, ay = 0.0f;
            const int ion = sp == 0, lec = sp == 1;
            switch (kind) {
            case 0: ax = p->ch; break;                                              /* tdens */
            case 1: if (ion) ax = p->ch; break;                                     /* idens */
            case 2: ax = p->u * gamprt * p->ch; ay = p->ch; break;                  /* tbetx */
            case 3: ax = p->v * gamprt * p->ch; ay = p->ch; break;                  /* tbety */
            case 4: ax = p->w * gamprt * p->ch; ay = p->ch; break;                  /* tbetz */
            case 5: if (ion) { ax = p->u * gamprt * p->ch; ay = p->ch; } break;     /* ibetx */
            case 6: if (ion) { ax = p->v * gamprt * p->ch; ay = p->ch; } break;     /* ibety */
            case 7: if (ion) { ax = p->w * gamprt * p->ch; ay = p->ch; } break;     /* ibetz */
            case 8: ax = p->u * p->ch; ay = p->ch; break;                           /* tmomx */
            case 9: ax = p->v * p->ch; ay = p->ch; break;                           /* tmomy */
            case 10: ax = p->w * p->ch; ay = p->ch; break;                          /* tmomz */
            case 11: if (ion) { ax = p->u * p->ch; ay = p->ch; } break;             /* imomx */
            case 12: if (ion) { ax = p->v * p->ch; ay = p->ch; } break;             /* imomy */
            case 13: if (ion) { ax = p->w * p->ch; ay = p->ch; } break;             /* imomz */
            case 14: if (lec) { ax = (1.0f / gamprt - 1.0f) * p->ch; ay = p->ch; } break; /* eener */
            case 15: if (ion) { ax = (1.0f / gamprt - 1.0f) * p->ch; ay = p->ch; } break; /* iener */
            default: break;
            }
            const int i = (int)p->x, j = (int)p->y, k = (int)p->z;
            int lz1 = k - idz > 1 ? k - idz : 1, lz2 = k + idz < s->mz ? k + idz : s->mz;
            if (s->dims == 2) { lz1 = 1; lz2 = 1; }
            const int ly1 = j - idy > 1 ? j - idy : 1, ly2 = j + idy < s->my ? j + idy : s->my;
            const int lx1 = i - idx > 1 ? i - idx : 1, lx2 = i + idx < s->mx ? i + idx : s->mx;
            for (int kk = lz1; kk <= lz2; kk++)
                for (int jj = ly1; jj <= ly2; jj++)
                    for (int ii = lx1; ii <= lx2; ii++) {
                        const int64_t l = (ii - 1) + iy * (jj - 1) + iz * (kk - 1);
                        cx[l] = cx[l] + ax;
                        cy[l] = cy[l] + ay;
                    }
        }
    }
    to_exchange_current(s);
    for (int k = 1; k <= s->mz; k++)
        for (int j = 1; j <= s->my; j++)
            for (int i = 1; i <= s->mx; i++) {
                int lz1 = k - idz > 1 ? k - idz : 1, lz2 = k + idz < s->mz ? k + idz : s->mz;
                if (s->dims == 2) { lz1 = 1; lz2 = 1; }
                const int ly1 = j - idy > 1 ? j - idy : 1, ly2 = j + idy < s->my ? j + idy : s->my;
                const int lx1 = i - idx > 1 ? i - idx : 1, lx2 = i + idx < s->mx ? i + idx : s->mx;
                const int64_t l = (i - 1) + iy * (j - 1) + iz * (k - 1);
                const float box = (float)((lx2 - lx1 + 1) * (ly2 - ly1 + 1) * (lz2 - lz1 + 1));
                cx[l] = cx[l] / box;
                cy[l] = cy[l] / box;
            }
    if (kind >= 2)
        for (int64_t l = 0; l < lot; l++) cx[l] = cy[l] != 0.0f ? cx[l] / cy[l] : 0.0f;
    memcpy(num, cx, sizeof(float) * lot);
    memcpy(den, cy, sizeof(float) * lot);
    memcpy(cx, keep, sizeof(float) * lot);
    memcpy(cy, keep + lot, sizeof(float) * lot);
    memcpy(cz, keep + 2 * lot, sizeof(float) * lot);
    free(keep);
}

/* ------------------------------------------------------------------------
 * Energy spectra in the flow frame per x-y slice (save_spectrum_2d,
 * code/output.F90:794-1249): gamma range over all particles, slice means
 * of the velocity, Lorentz transformation of each particle into its
 * slice's mean frame, histogram of log10(gamma' - 1) in gambins bins.
 * log10 of a single is evaluated in double (atanh series after splitting
 * off the binary exponent) and rounded once.
 * --------------------------------------------------------------------- */
float to_log10f(float x)
{
    if (!(x > 0.0f)) return x == 0.0f ? -INFINITY : NAN;
    if (isinf(x)) return x;
    int e;
    double m = frexp((double)x, &e); /* x = m 2^e, m in [0.5, 1) */
    if (m < 0.70710678118654752) {
        m = m * 2.0;
        e = e - 1;
    }
    const double s = (m - 1.0) / (m + 1.0), s2 = s * s;
    double t = 1.0 / 23.0;
    for (int k = 21; k >= 1; k -= 2) t = 1.0 / k + s2 * t;
    const double ln = 2.0 * s * t + (double)e * 0.69314718055994530942;
    return (float)(ln / 2.30258509299404568402);
}

int to_spectrum_dims(const to_state *s, int gambins, int *nx, int *ny)
{
    const int ng = s->nghost;
    const int mxmin = (int)((float)(s->mx - ng) * 0.5f) - 1200 + (ng / 2 + 1);
    const int mxmax = (int)((float)(s->mx - ng) * 0.5f) + 400 + (ng / 2 + 1);
    const int mymin = ng / 2 + 1, mymax = s->my - ng / 2;
    *nx = (mxmax - mxmin) / 30 > 1 ? (mxmax - mxmin) / 30 : 1;
    *ny = (mymax - mymin) / 30 > 1 ? (mymax - mymin) / 30 : 1;
    return gambins;
}

/* spec_i / spec_e: nxbins*nybins*gambins (x fastest); xgamma: gambins;
   xslice / yslice: nxbins / nybins; returns gammin and gammax */
/* save_spectrum (code/output.F90:380-785): x slices of about 100 cells over
   [3, mx0 - 2], lab-frame and mean-flow-frame spectra per species, weights
   splitratio^(1 - splitlev) ch (splitratio = 10, code/particles.F90:336),
   each bin divided by its gamma - 1. The electron loops start at p(maxhlf)
   as the reference's do (one record before the first electron). */
int to_spectrum_x_bins(const to_state *s)
{
    const int nb = (s->mx - 2 - 3) / 100;
    return nb > 1 ? nb : 1;
}

void to_spectrum_x(const to_state *s, int gambins, float *spec_i, float *spec_e, float *rest_i, float *rest_e,
                   float *xgamma, float *xslice, float *gmin_out, float *gmax_out)
{
    const int mxmin = 3, mxmax = s->mx - 2;
    const int nbins = to_spectrum_x_bins(s);
    const float dxslice = 1.0f * (float)(mxmax - mxmin) / (float)nbins;
    for (int i = 1; i <= nbins; i++) xslice[i - 1] = dxslice * (float)(i - 1) + 0.5f * dxslice + (float)mxmin;
    float gammin = 1.0f, gammax = 1.0f;
    for (int sp = 0; sp < 2; sp++) {
        const int64_t base = sp == 0 ? 0 : s->maxhlf, cnt = sp == 0 ? s->ions : s->lecs;
        for (int64_t n = 0; n < cnt; n++) {
            const to_particle *p = &s->p[base + n];
            const float gam = sqrtf(1.0f + (p->u * p->u + p->v * p->v + p->w * p->w));
            if (gam > gammax) gammax = gam;
            if (gam < gammin) gammin = gam;
        }
    }
    gammin = fmaxf(gammin, 1.0f + 1e-6f);
    const float lg0 = to_log10f(gammin - 1.0f);
    const float dgam = (to_log10f(gammax - 1.0f) - lg0) / (float)gambins;
    for (int i = 1; i <= gambins; i++) xgamma[i - 1] = powf(10.0f, (float)(i - 1) * dgam + lg0);
    float *um = calloc((size_t)nbins * 4, sizeof(float));
    float *vm = um + nbins, *wm = vm + nbins, *nd = wm + nbins;
    for (int sp = 0; sp < 2; sp++) {
        float *lab = sp == 0 ? spec_i : spec_e, *rest = sp == 0 ? rest_i : rest_e;
        memset(lab, 0, sizeof(float) * (size_t)nbins * gambins);
        memset(rest, 0, sizeof(float) * (size_t)nbins * gambins);
        memset(um, 0, sizeof(float) * (size_t)nbins * 4);
        /* ions: p(1..ions); electrons: p(maxhlf..maxhlf+lecs) */
        const int64_t first = sp == 0 ? 0 : s->maxhlf - 1, last = sp == 0 ? s->ions : s->maxhlf + s->lecs;
        for (int pass = 0; pass < 2; pass++) {
            for (int64_t n = first; n < last; n++) {
                const to_particle *p = &s->p[n];
                const float fxb = (p->x + (float)s->mxcum - (float)mxmin) / dxslice + 1.0f;
                if (!(fxb >= 1.0f)) continue;
                const int xbin = (int)fxb;
                if (xbin > nbins) continue;
                const int64_t sl = xbin - 1;
                const float w = powf(10.0f, 1.0f - (float)p->splitlev);
                const float gam = sqrtf(1.0f + (p->u * p->u + p->v * p->v + p->w * p->w));
                if (pass == 0) {
                    nd[sl] = nd[sl] + w * p->ch;
                    um[sl] = um[sl] + (p->u / gam) * w * p->ch;
                    vm[sl] = vm[sl] + (p->v / gam) * w * p->ch;
                    wm[sl] = wm[sl] + (p->w / gam) * w * p->ch;
                    continue;
                }
                const float fl = (to_log10f(gam - 1.0f) - lg0) / dgam + 1.0f;
                if (fl >= 1.0f && fl < (float)gambins + 1.0f)
                    lab[sl + nbins * ((int)fl - 1)] = lab[sl + nbins * ((int)fl - 1)] + w * p->ch;
                const float vx = um[sl], vy = vm[sl], vz = wm[sl];
                const float vr = sqrtf(vx * vx + vy * vy + vz * vz);
                const float gvr = 1.0f / sqrtf(1.0f - vr * vr);
                const float vr2 = vr * vr;
                const float uprime = -vx * gvr * gam + (1.0f + (gvr - 1.0f) * (vx * vx) / vr2) * p->u +
                                     (gvr - 1.0f) * vx * vy / vr2 * p->v + (gvr - 1.0f) * vx * vz / vr2 * p->w;
                const float vprime = -vy * gvr * gam + (gvr - 1.0f) * vx * vy / vr2 * p->u +
                                     (1.0f + (gvr - 1.0f) * (vy * vy) / vr2) * p->v + (gvr - 1.0f) * vy * vz / vr2 * p->w;
                const float wprime = -vz * gvr * gam + (gvr - 1.0f) * vx * vz / vr2 * p->u +
                                     (gvr - 1.0f) * vy * vz / vr2 * p->v + (1.0f + (gvr - 1.0f) * (vz * vz) / vr2) * p->w;
                const float gp = sqrtf(1.0f + (uprime * uprime + vprime * vprime + wprime * wprime));
                const float fg = (to_log10f(gp - 1.0f) - lg0) / dgam + 1.0f;
                if (!(fg >= 1.0f && fg < (float)gambins + 1.0f)) continue;
                rest[sl + nbins * ((int)fg - 1)] = rest[sl + nbins * ((int)fg - 1)] + w * p->ch;
            }
            if (pass == 0)
                for (int64_t l = 0; l < nbins; l++) {
                    um[l] = um[l] / nd[l];
                    vm[l] = vm[l] / nd[l];
                    wm[l] = wm[l] / nd[l];
                }
        }
        for (int64_t t = 0; t < (int64_t)nbins * gambins; t++) {
            lab[t] = lab[t] / xgamma[t / nbins];
            rest[t] = rest[t] / xgamma[t / nbins];
        }
    }
    free(um);
    *gmin_out = gammin;
    *gmax_out = gammax;
}

void to_spectrum_2d(const to_state *s, int gambins, float *spec_i, float *spec_e, float *xgamma, float *xslice,
                    float *yslice, float *gmin_out, float *gmax_out)
{
    const int ng = s->nghost;
    const int mxmin = (int)((float)(s->mx - ng) * 0.5f) - 1200 + (ng / 2 + 1);
    const int mxmax = (int)((float)(s->mx - ng) * 0.5f) + 400 + (ng / 2 + 1);
    const int mymin = ng / 2 + 1, mymax = s->my - ng / 2;
    int nxb, nyb;
    to_spectrum_dims(s, gambins, &nxb, &nyb);
    const float dxslice = 1.0f * (float)(mxmax - mxmin) / (float)nxb;
    const float dyslice = 1.0f * (float)(mymax - mymin) / (float)nyb;
    for (int i = 1; i <= nxb; i++) xslice[i - 1] = dxslice * (float)(i - 1) + 0.5f * dxslice + (float)mxmin;
    for (int i = 1; i <= nyb; i++) yslice[i - 1] = dyslice * (float)(i - 1) + 0.5f * dyslice + (float)mymin;
    float gammin = 1.0f, gammax = 1.0f;
    for (int sp = 0; sp < 2; sp++) {
        const int64_t base = sp == 0 ? 0 : s->maxhlf, cnt = sp == 0 ? s->ions : s->lecs;
        for (int64_t n = 0; n < cnt; n++) {
            const to_particle *p = &s->p[base + n];
            const float gam = sqrtf(1.0f + (p->u * p->u + p->v * p->v + p->w * p->w));
            if (gam > gammax) gammax = gam;
            if (gam < gammin) gammin = gam;
        }
    }
    gammin = fmaxf(gammin, 1.0f + 1e-6f);
    const float dgam = (to_log10f(gammax - 1.0f) - to_log10f(gammin - 1.0f)) / (float)gambins;
    for (int i = 1; i <= gambins; i++)
        xgamma[i - 1] = powf(10.0f, (float)(i - 1) * dgam + to_log10f(gammin - 1.0f));
    const int64_t nsl = (int64_t)nxb * nyb;
    float *um = calloc((size_t)nsl * 4, sizeof(float));
    float *vm = um + nsl, *wm = vm + nsl, *nd = wm + nsl;
    for (int sp = 0; sp < 2; sp++) {
        float *spec = sp == 0 ? spec_i : spec_e;
        memset(spec, 0, sizeof(float) * (size_t)nsl * gambins);
        memset(um, 0, sizeof(float) * (size_t)nsl * 4);
        const int64_t base = sp == 0 ? 0 : s->maxhlf, cnt = sp == 0 ? s->ions : s->lecs;
        for (int pass = 0; pass < 2; pass++) {
            for (int64_t n = 0; n < cnt; n++) {
                const to_particle *p = &s->p[base + n];
                if (p->ind <= 0) continue;
                const float fxb = (p->x + (float)s->mxcum - (float)mxmin) / dxslice + 1.0f;
                const float fyb = (p->y + (float)s->mycum - (float)mymin) / dyslice + 1.0f;
                if (!(fxb >= 1.0f && fyb >= 1.0f)) continue;
                const int xbin = (int)fxb, ybin = (int)fyb;
                if (xbin > nxb || ybin > nyb) continue;
                const int64_t sl = (xbin - 1) + (int64_t)nxb * (ybin - 1);
                const float gam = sqrtf(1.0f + (p->u * p->u + p->v * p->v + p->w * p->w));
                if (pass == 0) {
                    nd[sl] = nd[sl] + p->ch;
                    um[sl] = um[sl] + (p->u / gam) * p->ch;
                    vm[sl] = vm[sl] + (p->v / gam) * p->ch;
                    wm[sl] = wm[sl] + (p->w / gam) * p->ch;
                    continue;
                }
                const float vx = um[sl], vy = vm[sl], vz = wm[sl];
                const float vr = sqrtf(vx * vx + vy * vy + vz * vz);
                const float gvr = 1.0f / sqrtf(1.0f - vr * vr);
                const float vr2 = vr * vr;
                const float uprime = -vx * gvr * gam + (1.0f + (gvr - 1.0f) * (vx * vx) / vr2) * p->u +
                                     (gvr - 1.0f) * vx * vy / vr2 * p->v + (gvr - 1.0f) * vx * vz / vr2 * p->w;
                const float vprime = -vy * gvr * gam + (gvr - 1.0f) * vx * vy / vr2 * p->u +
                                     (1.0f + (gvr - 1.0f) * (vy * vy) / vr2) * p->v + (gvr - 1.0f) * vy * vz / vr2 * p->w;
                const float wprime = -vz * gvr * gam + (gvr - 1.0f) * vx * vz / vr2 * p->u +
                                     (gvr - 1.0f) * vy * vz / vr2 * p->v + (1.0f + (gvr - 1.0f) * (vz * vz) / vr2) * p->w;
                const float gp = sqrtf(1.0f + (uprime * uprime + vprime * vprime + wprime * wprime));
                const float fg = (to_log10f(gp - 1.0f) - to_log10f(gammin - 1.0f)) / dgam + 1.0f;
                if (!(fg >= 1.0f && fg < (float)gambins + 1.0f)) continue;
                const int gbin = (int)fg;
                spec[sl + nsl * (gbin - 1)] = spec[sl + nsl * (gbin - 1)] + p->ch;
            }
            if (pass == 0)
                for (int64_t l = 0; l < nsl; l++) {
                    um[l] = um[l] / nd[l];
                    vm[l] = vm[l] / nd[l];
                    wm[l] = wm[l] / nd[l];
                }
        }
    }
    free(um);
    *gmin_out = gammin;
    *gmax_out = gammax;
}

/* ------------------------------------------------------------------------
 * output_tot (code/output.F90:2494-3884): one .tot. variable sampled every
 * istep nodes; E and B through interpolfld (code/output.F90:4995-5127).
 * --------------------------------------------------------------------- */
static void to_out_axis(int m, int64_t cum, int istep, int *start, int *n)
{
    int s = 1, f = m;
    while (s <= m && (((s + cum) % istep) + istep) % istep != 0) s++;
    while (f >= 1 && (((f + cum) % istep) + istep) % istep != 0) f--;
    *start = s;
    *n = f >= s ? (f - s) / istep + 1 : 0;
}

int to_output_dims(const to_state *s, int istep, int *dims)
{
    int st;
    to_out_axis(s->mx, s->mxcum, istep, &st, &dims[0]);
    to_out_axis(s->my, s->mycum, istep, &st, &dims[1]);
    if (s->dims == 3) to_out_axis(s->mz, s->mzcum, istep, &st, &dims[2]);
    else dims[2] = 1;
    return dims[0] * dims[1] * dims[2];
}

/* interpolfld for one component: a(l + o) with l the reference's 1-based
   linear index of the (clamped) node */
static float to_interpolfld(const to_state *s, int comp, const float *a, float x, float y, float z)
{
    int i = (int)x, j = (int)y, k = (int)z;
    float dx = x - (float)i, dy = y - (float)j, dz = z - (float)k;
    if (i == 1) i = 2;
    if (i == s->mx) i = s->mx - 1;
    if (j == 1) j = 2;
    if (j == s->my) j = s->my - 1;
    if (k == 1) k = 2;
    if (k == s->mz) k = s->mz - 1;
    int64_t ix = 1, iy = s->mx, iz = (int64_t)s->mx * s->my;
    if (s->dims == 2) {
        k = 1;
        dz = 0.0f;
        iz = 0;
    }
    const float *L = a + (i - 1) + iy * (j - 1) + iz * (k - 1);
#define A(o) L[(o)]
    float f, g;
    if (comp == 0) {
        f = A(0) + A(-ix) + dx * (A(ix) - A(-ix));
        f = f + dy * (A(iy) + A(-ix + iy) + dx * (A(ix + iy) - A(-ix + iy)) - f);
        g = A(iz) + A(-ix + iz) + dx * (A(ix + iz) - A(-ix + iz));
        g = g + dy * (A(iy + iz) + A(-ix + iy + iz) + dx * (A(ix + iy + iz) - A(-ix + iy + iz)) - g);
        return (f + dz * (g - f)) * 0.5f;
    }
    if (comp == 1) {
        f = A(0) + A(-iy) + dy * (A(iy) - A(-iy));
        f = f + dz * (A(iz) + A(-iy + iz) + dy * (A(iy + iz) - A(-iy + iz)) - f);
        g = A(ix) + A(-iy + ix) + dy * (A(iy + ix) - A(-iy + ix));
        g = g + dz * (A(iz + ix) + A(-iy + iz + ix) + dy * (A(iy + iz + ix) - A(-iy + iz + ix)) - g);
        return (f + dx * (g - f)) * 0.5f;
    }
    if (comp == 2) {
        f = A(0) + A(-iz) + dz * (A(iz) - A(-iz));
        f = f + dx * (A(ix) + A(-iz + ix) + dz * (A(iz + ix) - A(-iz + ix)) - f);
        g = A(iy) + A(-iz + iy) + dz * (A(iz + iy) - A(-iz + iy));
        g = g + dx * (A(ix + iy) + A(-iz + ix + iy) + dz * (A(iz + ix + iy) - A(-iz + ix + iy)) - g);
        return (f + dy * (g - f)) * 0.5f;
    }
    if (comp == 3) {
        f = A(-iy) + A(-iy - iz) + dz * (A(-iy + iz) - A(-iy - iz));
        f = A(0) + A(-iz) + dz * (A(iz) - A(-iz)) + f + dy * (A(iy) + A(iy - iz) + dz * (A(iy + iz) - A(iy - iz)) - f);
        g = A(ix - iy) + A(ix - iy - iz) + dz * (A(ix - iy + iz) - A(ix - iy - iz));
        g = A(ix) + A(ix - iz) + dz * (A(ix + iz) - A(ix - iz)) + g +
            dy * (A(ix + iy) + A(ix + iy - iz) + dz * (A(ix + iy + iz) - A(ix + iy - iz)) - g);
        return (f + dx * (g - f)) * 0.25f;
    }
    if (comp == 4) {
        f = A(-iz) + A(-iz - ix) + dx * (A(-iz + ix) - A(-iz - ix));
        f = A(0) + A(-ix) + dx * (A(ix) - A(-ix)) + f + dz * (A(iz) + A(iz - ix) + dx * (A(iz + ix) - A(iz - ix)) - f);
        g = A(iy - iz) + A(iy - iz - ix) + dx * (A(iy - iz + ix) - A(iy - iz - ix));
        g = A(iy) + A(iy - ix) + dx * (A(iy + ix) - A(iy - ix)) + g +
            dz * (A(iy + iz) + A(iy + iz - ix) + dx * (A(iy + iz + ix) - A(iy + iz - ix)) - g);
        return (f + dy * (g - f)) * 0.25f;
    }
    f = A(-ix) + A(-ix - iy) + dy * (A(-ix + iy) - A(-ix - iy));
    f = A(0) + A(-iy) + dy * (A(iy) - A(-iy)) + f + dx * (A(ix) + A(ix - iy) + dy * (A(ix + iy) - A(ix - iy)) - f);
    g = A(iz - ix) + A(iz - ix - iy) + dy * (A(iz - ix + iy) - A(iz - ix - iy));
    g = A(iz) + A(iz - iy) + dy * (A(iz + iy) - A(iz - iy)) + g +
        dx * (A(iz + ix) + A(iz + ix - iy) + dy * (A(iz + ix + iy) - A(iz + ix - iy)) - g);
    return (f + dz * (g - f)) * 0.25f;
#undef A
}

/* var: 0-5 E, B; 6-8 currents; 16 + k the meanq_fld_cur moment k */
int to_output_var(to_state *s, int var, int istep, int idx, int idy, int idz, float *out)
{
    int st[3], n[3];
    to_out_axis(s->mx, s->mxcum, istep, &st[0], &n[0]);
    to_out_axis(s->my, s->mycum, istep, &st[1], &n[1]);
    if (s->dims == 3) to_out_axis(s->mz, s->mzcum, istep, &st[2], &n[2]);
    else {
        st[2] = 1;
        n[2] = 1;
    }
    const int64_t lot = to_lot(s);
    float *num = NULL, *den = NULL;
    const float *src;
    float *arrs[9] = {s->ex, s->ey, s->ez, s->bx, s->by, s->bz, s->curx, s->cury, s->curz};
    if (var >= 16) {
        num = malloc(sizeof(float) * lot);
        den = malloc(sizeof(float) * lot);
        to_meanq(s, var - 16, idx, idy, idz, num, den);
        src = num;
    } else {
        src = arrs[var];
    }
    int64_t t = 0;
    for (int c = 0; c < n[2]; c++)
        for (int b = 0; b < n[1]; b++)
            for (int a = 0; a < n[0]; a++, t++) {
                const int i = st[0] + istep * a, j = st[1] + istep * b, k = s->dims == 3 ? st[2] + istep * c : 1;
                if (var < 6) {
                    const float e = s->external_fields ? s->ext[var] : 0.0f;
                    out[t] = to_interpolfld(s, var, src, (float)i, (float)j, (float)k) + e;
                } else {
                    out[t] = src[(i - 1) + (int64_t)s->mx * (j - 1) + (int64_t)s->mx * s->my * (k - 1)];
                }
            }
    free(num);
    free(den);
    return (int)t;
}

/* output_tot's particle sample (prtl.tot, code/output.F90:3293-3884): the
   species' particles with modulo(ind / 2, stride) = 0 in array order;
   vals[k * cap + i] = x + mxcum, y + mycum, z + mzcum, u, v, w, ch, gamma;
   ids[k * cap + i] = ind, proc. Returns the number selected (vals and ids
   are written only when it fits in cap). */
int64_t to_output_particles(const to_state *s, int species, int stride, int64_t cap, float *vals, int32_t *ids)
{
    const int64_t base = species == 0 ? 0 : s->maxhlf, cnt = species == 0 ? s->ions : s->lecs;
    int64_t total = 0;
    for (int64_t n = 0; n < cnt; n++) {
        const int h = s->p[base + n].ind / 2;
        if (((h % stride) + stride) % stride == 0) total++;
    }
    if (total > cap) return total;
    int64_t o = 0;
    for (int64_t n = 0; n < cnt; n++) {
        const to_particle *p = &s->p[base + n];
        const int h = p->ind / 2;
        if (((h % stride) + stride) % stride != 0) continue;
        vals[o] = p->x + (float)s->mxcum;
        vals[cap + o] = p->y + (float)s->mycum;
        vals[2 * cap + o] = p->z + (float)s->mzcum;
        vals[3 * cap + o] = p->u;
        vals[4 * cap + o] = p->v;
        vals[5 * cap + o] = p->w;
        vals[6 * cap + o] = p->ch;
        vals[7 * cap + o] = sqrtf(1.0f + (p->u * p->u + p->v * p->v + p->w * p->w));
        ids[o] = p->ind;
        ids[cap + o] = p->proc;
        o++;
    }
    return total;
}

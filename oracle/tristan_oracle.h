/*
 * CPU oracle for the TRISTAN-MP per-step PIC hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the oracle: the tests, the
 * smoke check and the CPU-baseline leg of bench.py call it to produce the
 * reference answer. The GPU product path never links, loads or calls it.
 *
 * It restates, routine by routine and in the reference's floating-point
 * operation order, the Fortran subroutines of
 * mrowan137/tristan-mp-pu-master_densdecomp that make up one time step
 * (code/tristanmainloop.F90:107-344): the Boris movers, the Esirkepov
 * current deposits, the deposit driver's periodic wrap / discard /
 * compaction, the Yee B and E advances, the ghost-layer copies, the current
 * ghost fold, the binomial current filter, add_current and the per-cell
 * counting-sort reorder.
 *
 * Parity pin: the reference ships no tests, fixtures or golden vectors and
 * no Fortran compiler is available to run it, so this restatement is
 * "parity unpinned" against reference outputs. It is pinned instead by
 * (a) an independent pure-Python transliteration of the same Fortran
 * (tests/golden/make_golden.py) that must agree bit for bit, and
 * (b) physics known-answer tests (shape partition of unity, per-particle
 * discrete charge continuity of the Esirkepov current, Yee vacuum
 * dispersion with the Corr factor, Gauss's law under the filter).
 *
 * Arrays use the reference's Fortran layout: field(mx,my,mz), x fastest,
 * 0-based linear index l = (i-1) + mx*(j-1) + mx*my*(k-1) for the 1-based
 * Fortran cell (i,j,k). Particles use the reference's 40-byte record
 * (code/particles.F90:51-55). Ions occupy p[0 .. ions-1], electrons
 * p[maxhlf .. maxhlf+lecs-1] (code/particles.F90:303-304).
 *
 * Build: gcc -O2 -ffp-contract=off (no FMA contraction, no fast-math), so
 * every float operation rounds exactly once, as the GPU kernels do.
 */
#ifndef TRISTAN_ORACLE_H
#define TRISTAN_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* one particle, field for field the reference's `type particle` */
typedef struct {
    float x, y, z, u, v, w, ch;
    int32_t ind, proc, splitlev;
} to_particle;

/* quirk switches (bit flags in to_state.quirks) */
#define TO_QUIRK_Q5_LHS 1 /* fold row `nghost` of cury with curx(:,my) as the
                             shape-mismatched assignment at
                             code/fieldboundaries.F90:1938 does when the
                             compiler loops over the left-hand side's extent */

typedef struct {
    /* grid: full extents including ghosts (2D: mz = 1) */
    int32_t dims, order;
    int32_t mx, my, mz;
    int32_t nghost, nghostz;
    int32_t periodic[3];
    int32_t ntimes;
    int32_t quirks;
    /* physics constants exactly as code/particles.F90:219-233 derives them */
    float c, corr, qi, qe, qmi, qme;
    /* external constant fields added in the mover when external_fields != 0
       (get_external_fields hook, user/user_weibel.F90:172-183) */
    int32_t external_fields;
    float ext[6]; /* ex, ey, ez, bx, by, bz */
    /* open-boundary window (allocate_particles, code/particles.F90:335-340);
       used only along non-periodic axes */
    double x1in, x2in, y1in, y2in, z1in, z2in;
    int64_t mxcum, mycum, mzcum;
    /* deposit mode: 0 = FP32 accumulation in the reference's order,
       1 = int64 fixed point, each contribution rounded to 2^-fx_shift */
    int32_t fixed;
    int32_t fx_shift;
    /* particles */
    int64_t maxhlf;
    int64_t ions, lecs;
    int64_t lap, lapreorder;
    to_particle *p;      /* 2*maxhlf records */
    to_particle *tempp;  /* maxhlf records (reorder scratch) */
    int32_t *pind;       /* maxhlf flags (deposit compaction) */
    int32_t *pall;       /* mx*my*mz+1 counters (reorder) */
    /* fields, mx*my*mz floats each */
    float *ex, *ey, *ez, *bx, *by, *bz;
    float *curx, *cury, *curz;
    float *temp;
    int64_t *fx, *fy, *fz; /* fixed-point accumulators (fixed != 0) */
    /* statistics of the last deposit call */
    int64_t nionout, nlecout;
} to_state;

/* lengths */
int64_t to_lot(const to_state *s);

/* movers: code/particles_movedeposit.F90:63-88 (move_particles) */
void to_move_particles(to_state *s);
void to_mover(to_state *s, int64_t n1, int64_t n2, float qm); /* 0-based [n1,n2) */

/* deposit driver: code/particles_movedeposit.F90:1281-2051 */
void to_deposit_particles(to_state *s);
/* one particle's Esirkepov deposit (densdecomp_{1,2,3}ord,
   code/particles.F90:678-1358); q is the particle charge */
void to_densdecomp(to_state *s, float x2, float y2, float z2,
                   float x1, float y1, float z1, float q);
/* fixed-point accumulators -> float currents */
void to_fixed_to_float(to_state *s);

/* fields: code/fields.F90 */
void to_reset_currents(to_state *s);     /* :499-506 */
void to_advance_b_halfstep(to_state *s); /* :586-728 */
void to_advance_e_fullstep(to_state *s); /* :739-870 */
void to_add_current(to_state *s);        /* :1372-1395 */

/* boundaries: code/fieldboundaries.F90 */
void to_bc_b1(to_state *s);              /* :181-263 */
void to_bc_e1(to_state *s);              /* :306-392 */
void to_exchange_current(to_state *s);   /* :1768-2189 */
void to_apply_filter1_opt(to_state *s);  /* code/filter.F90:8-221 */

/* reorder: code/particles.F90:394-497 */
void to_reorder_particles(to_state *s);  /* cadence wrapper */
void to_reorder_particles_(to_state *s); /* the stable counting sort */

/* one lap of mainloop (code/tristanmainloop.F90:107-344) for the periodic
   problems: field BCs, B half step, mover, B half step, E step, deposit,
   fold, filter, add_current, reorder cadence */
void to_step(to_state *s);

/* FP64 diagnostics */
typedef struct {
    double gauss_residual;   /* ||div E - F^ntimes(rho)||_2 / ||F^ntimes(rho)||_2 */
    double gauss_abs;        /* ||div E - F^ntimes(rho)||_2 */
    double rho_norm;         /* ||F^ntimes(rho)||_2 */
    double e_field;          /* sum over interior of (E^2)/2 */
    double e_mag;            /* sum over interior of (B^2)/2 */
    double e_kin_ions;       /* sum over ions of (gamma-1)*|m| */
    double e_kin_lecs;
    double p_part[3];        /* sum m*u over all particles */
    double p_field[3];       /* sum E x B over the interior */
    double charge_total;     /* sum of rho over the interior */
} to_diag;

/* charge density on nodes with the same B-spline used by the deposit,
   folded periodically and filtered ntimes; FP64 */
void to_charge_density(const to_state *s, double *rho);
void to_diagnostics(const to_state *s, to_diag *out);

/* threads used by the OpenMP build (1 in the serial build) */
int to_num_threads(void);

/* ------------------------------------------------------------------------
 * Collisionless-shock setup, 2D (user_pu/user_shock_pu.F90): reflecting
 * left wall with zigzag partial deposits, conductor behind the wall and
 * right-edge field reset, moving injector; the Park-Miller generator
 * (code/aux.F90:82-134) and the Maxwell-Juttner loader
 * (code/particles.F90:2126-2273, :2439-2938).
 * --------------------------------------------------------------------- */
#define TO_PDF_SZ 1000

typedef struct {
    /* left wall (particle_bc_user, user_shock_pu.F90:514-611) */
    int32_t wall;
    double walloc;          /* wall position (global x) */
    float gammawall, betawall;
    /* field_bc_user (user_shock_pu.F90:460-488): ey = ez = 0 on local
       i = cond_i1..cond_i2, and the upstream fields written on
       i = edge_i1..edge_i2 */
    int32_t cond_i1, cond_i2, edge_i1, edge_i2;
    float edge[6];          /* ex ey ez bx by bz */
    /* moving injector (inject_particles_user, :364-395) */
    int32_t inject;
    double xinject2;
    float betainj;
    double xinj_max;        /* mx0 - 15 */
    float ppc0, gamma_drift, weight;
    float y1, y2;           /* injection band, global y */
    /* Maxwell-Juttner loader */
    float pcosthmult;
    int32_t sigma_nonzero;
    float gamma_table_i[TO_PDF_SZ], pdf_table_i[TO_PDF_SZ + 1];
    float gamma_table_e[TO_PDF_SZ], pdf_table_e[TO_PDF_SZ + 1];
    double dseed;
    int32_t totalpartnum;
    int64_t injected;       /* pairs injected by the last call */
} to_shock;

float to_random(double *dseed);                                   /* aux.F90:82-99 */
float to_poisson(float numps, double *dseed);                     /* aux.F90:110-134 */
void to_init_maxw_table(float delgam, int dims, float pcosthmult, float *gamma_table, float *pdf_table);
void to_maxwell_dist(float gamma0, float cd, double *dseed, float *u, float *v, float *w,
                     const float *gamma_table, const float *pdf_table, float pcosthmult, int sigma_nonzero);
/* inject_plasma_region, drift along x (direction 1); the 3D form takes the
   z range (code/particles.F90:2695-2728) */
void to_inject_plasma_region(to_state *s, to_shock *k, float x1, float x2, float y1, float y2, float ppc,
                             float weight);
void to_inject_plasma_region3(to_state *s, to_shock *k, float x1, float x2, float y1, float y2, float z1, float z2,
                              float ppc, float weight);
void to_inject_particles_user(to_state *s, to_shock *k);          /* :364-395 */
void to_particle_bc_user(to_state *s, to_shock *k);               /* :514-611 */
void to_field_bc_user(to_state *s, const to_shock *k);            /* :460-488 */
/* the shock's lap: the periodic lap with the user hooks at their places
   in code/tristanmainloop.F90:117-303 */
void to_step_shock(to_state *s, to_shock *k);
/* grid moments of meanq_fld_cur (code/output.F90:5222-5482); kind 0..15 =
   tdens idens tbetx tbety tbetz ibetx ibety ibetz tmomx tmomy tmomz imomx
   imomy imomz eener iener; num receives the moment, den the box-averaged
   weight (both mx*my*mz); the current arrays are left as they were */
void to_meanq(to_state *s, int kind, int idx, int idy, int idz, float *num, float *den);
/* output_tot (code/output.F90:2494-3884): the istep-sampled counts, and one
   variable (0-5 E/B through interpolfld, 6-8 currents, 16 + k moment k) */
int to_output_dims(const to_state *s, int istep, int *dims);
int to_output_var(to_state *s, int var, int istep, int idx, int idy, int idz, float *out);
/* output_tot's particle sample (prtl.tot): selected count; values when it
   fits in cap */
int64_t to_output_particles(const to_state *s, int species, int stride, int64_t cap, float *vals, int32_t *ids);
/* flow-frame energy spectra per slice (save_spectrum_2d,
   code/output.F90:794-1249); dims from to_spectrum_dims */
float to_log10f(float x);
int to_spectrum_dims(const to_state *s, int gambins, int *nx, int *ny);
/* save_spectrum (code/output.F90:380-785): x slices, lab-frame and
   flow-frame spectra, divided by gamma - 1 */
int to_spectrum_x_bins(const to_state *s);
void to_spectrum_x(const to_state *s, int gambins, float *spec_i, float *spec_e, float *rest_i, float *rest_e,
                   float *xgamma, float *xslice, float *gmin_out, float *gmax_out);
void to_spectrum_2d(const to_state *s, int gambins, float *spec_i, float *spec_e, float *xgamma, float *xslice,
                    float *yslice, float *gmin_out, float *gmax_out);
/* sin and cos of a float argument, evaluated in double and rounded once */
void to_sincosf(float x, float *sn, float *cs);

#ifdef __cplusplus
}
#endif
#endif
